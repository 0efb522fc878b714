// C ABI of the GB300 tracer (include/omg_cuda.h), part 6: the reference's
// wire formats.
//
// - The web bridge's flat trace jobs (crates/omg-web/src/lib.rs:150-202 box
//   jobs, :365-416 world jobs), decoded the way its GPU driver reads them
//   (web/gpu.js:181-199, 420-437), traced as one batch, and returned as the
//   driver's injection records (lib.rs:204-218).
// - ParamBlock's flat f32 layout (crates/omg-core/src/params.rs:66-141).
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "runtime.h"

namespace {

// JavaScript's ToUint32 of a Number: what gpu.js gets when it stores a job
// word into a Uint32Array slot (u32[3] = f[o + 1], gpu.js:186-188).
uint32_t js_to_u32(float f) {
  if (!std::isfinite(f)) return 0u;
  double m = std::fmod(std::trunc((double)f), 4294967296.0);
  if (m < 0.0) m += 4294967296.0;
  return (uint32_t)m;
}

// Rust's `f32 as u32` / `as u64` / `as usize`: truncation, saturating, NaN -> 0.
template <class U>
U rust_as(float f) {
  if (!(f > 0.0f)) return 0;
  const double d = std::trunc((double)f);
  if (d >= (double)std::numeric_limits<U>::max()) return std::numeric_limits<U>::max();
  return (U)d;
}

void material3(omg_material& m, const float* absorption, float scattering, const float* transmission) {
  std::memset(&m, 0, sizeof(m));
  for (int b = 0; b < 3; b++) {
    m.absorption[b] = absorption[b];
    m.transmission[b] = transmission[b];
  }
  m.scattering = scattering;
}

// Trace the decoded jobs and lay the results out as injection records:
// per job n_bins x 3 bins, then n_bins x 3 dirs.
int32_t trace_to_echo(omg_ctx* ctx, const std::vector<omg_job>& jobs, const std::vector<omg_panel>& panels,
                      float* echo, omg_reverb* reverb) {
  const size_t nb = ctx->prm.n_bins, n = jobs.size();
  std::vector<float> bins(n * nb * 3), dirs(n * nb * 3);
  const int32_t rc = omg_trace_batch(ctx, jobs.data(), (uint32_t)n, panels.empty() ? nullptr : panels.data(),
                                     (uint32_t)panels.size(), bins.data(), dirs.data(), reverb);
  if (rc != OMG_OK) return rc;
  for (size_t j = 0; j < n; j++) {
    float* o = echo + j * nb * 6;
    std::memcpy(o, &bins[j * nb * 3], nb * 3 * sizeof(float));
    std::memcpy(o + nb * 3, &dirs[j * nb * 3], nb * 3 * sizeof(float));
  }
  return OMG_OK;
}

}  // namespace

int32_t omg_trace_web_box_jobs(omg_ctx* ctx, const float* jobs, uint32_t n_floats, float* echo, uint32_t* ids,
                               omg_reverb* reverb) {
  if (!ctx || !jobs || !echo || n_floats == 0 || n_floats % OMG_WEB_BOX_JOB_F32S != 0 || ctx->prm.n_bands != 3)
    return OMG_E_INVALID;
  const uint32_t n = n_floats / OMG_WEB_BOX_JOB_F32S;
  std::vector<omg_job> js(n);
  for (uint32_t i = 0; i < n; i++) {
    const float* f = jobs + (size_t)i * OMG_WEB_BOX_JOB_F32S;
    omg_job& j = js[i];
    std::memset(&j, 0, sizeof(j));
    j.geom = OMG_GEOM_BOX;
    j.n_rays = js_to_u32(f[1]);
    j.seed = js_to_u32(f[2]);
    for (int k = 0; k < 3; k++) {
      j.box_size[k] = f[3 + k];
      j.src[k] = f[6 + k];
      j.lis[k] = f[9 + k];
      j.energy[k] = f[12 + k];
    }
    for (int w = 0; w < 6; w++) {
      const float* m = f + 15 + 7 * w;  // absorption x3, scattering, transmission x3
      material3(j.box_walls[w], m, m[3], m + 4);
    }
    if (ids) ids[i] = js_to_u32(f[0]);
  }
  return trace_to_echo(ctx, js, {}, echo, reverb);
}

int32_t omg_trace_web_world_jobs(omg_ctx* ctx, uint32_t scene_id, const float* jobs, uint32_t n_floats,
                                 float* echo, uint32_t* ids, omg_reverb* reverb) {
  if (!ctx || !jobs || !echo || n_floats == 0 || n_floats % OMG_WEB_WORLD_JOB_F32S != 0 ||
      ctx->prm.n_bands != 3)
    return OMG_E_INVALID;
  const uint32_t n = n_floats / OMG_WEB_WORLD_JOB_F32S;
  std::vector<omg_job> js(n);
  std::vector<omg_panel> panels;
  for (uint32_t i = 0; i < n; i++) {
    const float* f = jobs + (size_t)i * OMG_WEB_WORLD_JOB_F32S;
    omg_job& j = js[i];
    std::memset(&j, 0, sizeof(j));
    j.geom = OMG_GEOM_MESH;
    j.scene_id = scene_id;
    j.n_rays = js_to_u32(f[1]);
    j.seed = js_to_u32(f[2]);
    for (int k = 0; k < 3; k++) {
      j.src[k] = f[3 + k];
      j.lis[k] = f[6 + k];
      j.energy[k] = 1.0f;  // gpu.js:434, unit energy
    }
    // Math.min(jobs[9], 64) panels (gpu.js:425)
    const float np_f = std::fmin(f[9], (float)OMG_WEB_WORLD_MAX_PANELS);
    const uint32_t np = np_f > 0.0f ? (uint32_t)np_f : 0u;
    j.panel_offset = (uint32_t)panels.size();
    j.n_panels = np;
    for (uint32_t p = 0; p < np; p++) {
      const float* q = f + 10 + 16 * p;  // min xyz, scattering, max xyz, 0, absorption xyz, 0, transmission xyz, 0
      omg_panel pn;
      std::memset(&pn, 0, sizeof(pn));
      for (int k = 0; k < 3; k++) {
        pn.mn[k] = q[k];
        pn.mx[k] = q[4 + k];
      }
      material3(pn.material, q + 8, q[3], q + 12);
      panels.push_back(pn);
    }
    if (ids) ids[i] = js_to_u32(f[0]);
  }
  return trace_to_echo(ctx, js, panels, echo, reverb);
}

// ---------------------------------------------------------------- ParamBlock
uint32_t omg_param_block_flat_len(uint32_t n_taps) {
  return OMG_PARAM_FLAT_HEADER + n_taps * OMG_PARAM_FLAT_PER_TAP;
}

int32_t omg_param_block_write_flat(const omg_param_block* pb, const omg_tap* taps, uint32_t n_taps, float* out,
                                   uint32_t out_len) {
  if (!pb || !out || (n_taps && !taps) || n_taps > (0xFFFFFFFFu - OMG_PARAM_FLAT_HEADER) / OMG_PARAM_FLAT_PER_TAP ||
      out_len < omg_param_block_flat_len(n_taps))
    return OMG_E_INVALID;
  const uint32_t len = omg_param_block_flat_len(n_taps);
  std::memset(out, 0, (size_t)len * sizeof(float));
  out[0] = (float)pb->version;
  out[1] = (float)n_taps;
  for (int b = 0; b < 3; b++) {
    out[2 + b] = pb->rt60[b];
    out[5 + b] = pb->level[b];
  }
  if (pb->has_remote) {
    out[8] = 1.0f;
    for (int b = 0; b < 3; b++) {
      out[9 + b] = pb->remote_rt60[b];
      out[12 + b] = pb->remote_send[b];
    }
    std::memcpy(&out[15], pb->remote_sh, 9 * sizeof(float));
  }
  for (uint32_t i = 0; i < n_taps; i++) {
    float* o = out + OMG_PARAM_FLAT_HEADER + (size_t)i * OMG_PARAM_FLAT_PER_TAP;
    o[0] = (float)taps[i].key;
    o[1] = taps[i].delay_s;
    std::memcpy(&o[2], taps[i].dir, 3 * sizeof(float));
    std::memcpy(&o[5], taps[i].gains, 3 * sizeof(float));
  }
  return OMG_OK;
}

int32_t omg_param_block_read_flat(const float* data, uint32_t len, omg_param_block* pb, omg_tap* taps,
                                  uint32_t max_taps, uint32_t* n_taps) {
  if (!data || !pb || !n_taps || len < OMG_PARAM_FLAT_HEADER) return OMG_E_INVALID;
  const uint64_t nt = rust_as<uint64_t>(data[1]);
  *n_taps = nt > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)nt;
  if (nt > (uint64_t)(len - OMG_PARAM_FLAT_HEADER) / OMG_PARAM_FLAT_PER_TAP || nt > max_taps || (nt && !taps))
    return OMG_E_INVALID;
  std::memset(pb, 0, sizeof(*pb));
  pb->version = rust_as<uint64_t>(data[0]);
  for (int b = 0; b < 3; b++) {
    pb->rt60[b] = data[2 + b];
    pb->level[b] = data[5 + b];
  }
  if (data[8] > 0.5f) {
    pb->has_remote = 1;
    for (int b = 0; b < 3; b++) {
      pb->remote_rt60[b] = data[9 + b];
      pb->remote_send[b] = data[12 + b];
    }
    std::memcpy(pb->remote_sh, &data[15], 9 * sizeof(float));
  }
  for (uint64_t i = 0; i < nt; i++) {
    const float* o = data + OMG_PARAM_FLAT_HEADER + i * OMG_PARAM_FLAT_PER_TAP;
    taps[i].key = rust_as<uint32_t>(o[0]);
    taps[i].delay_s = o[1];
    std::memcpy(taps[i].dir, &o[2], 3 * sizeof(float));
    std::memcpy(taps[i].gains, &o[5], 3 * sizeof(float));
  }
  return OMG_OK;
}

int32_t omg_param_block_from_late(const omg_late_state* states, uint32_t n, omg_param_block* out) {
  if ((n && (!states || !out))) return OMG_E_INVALID;
  for (uint32_t i = 0; i < n; i++) {
    std::memset(&out[i], 0, sizeof(out[i]));
    out[i].version = states[i].version;
    for (int b = 0; b < 3; b++) {
      out[i].rt60[b] = states[i].rt60[b];
      out[i].level[b] = states[i].level[b];
    }
  }
  return OMG_OK;
}
