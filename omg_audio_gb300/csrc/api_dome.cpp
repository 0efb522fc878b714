// C ABI of the GB300 tracer (include/omg_cuda.h), part 3: the ambient dome
// (DomeProbe, crates/omg-scene/src/dome.rs:293-478) for many listeners at once.
#include "runtime.h"

using namespace omg;

namespace omg {

struct DomeRec {
  uint32_t scene_id = 0;
  uint32_t n_fan = 0, nb = 3;
  std::vector<DDomePanel> glass;
  DevBuf<float4> fan;
  uint32_t eye_cap = 0;
  DevBuf<float> ema;          // eye_cap x 9 x nb
  DevBuf<uint32_t> primed;    // eye_cap
  // per-call scratch
  DevBuf<float> eyes, tp, raw, dir, energy;
  DevBuf<uint8_t> esc;
  DevBuf<DDomePanel> panels;
  DevBuf<DLaunch> hdr;
  DevBuf<uint32_t> events;
  cudaEvent_t done = nullptr;
  uint64_t last_events[2] = {0, 0};
  // pinned staging of a submitted sample (inputs up, results down)
  PinBuf<float> h_eyes, h_energy, h_dir, h_raw, h_tp;
  PinBuf<uint8_t> h_esc;
  PinBuf<DDomePanel> h_panels;
  PinBuf<DLaunch> h_hdr;
  PinBuf<uint32_t> h_events;
  bool pending = false;
  uint32_t p_eyes = 0, p_rays = 0, p_flags = 0;
  ~DomeRec() {
    if (done) cudaEventDestroy(done);
  }
};

}  // namespace omg

namespace {

DDomePanel to_dpanel(const omg_dome_panel& p, uint32_t nb) {
  DDomePanel d;
  std::memset(&d, 0, sizeof(d));
  d.axis = p.axis;
  d.plane = p.plane;
  d.lat0 = p.lat0;
  d.lat1 = p.lat1;
  d.z0 = p.z0;
  d.z1 = p.z1;
  d.glass = p.glass;
  for (uint32_t b = 0; b < nb; b++) d.t2[b] = p.trans[b] * p.trans[b];
  return d;
}

bool valid_dome_panel(const omg_dome_panel& p, uint32_t nb) {
  if (p.axis != 0 && p.axis != 1) return false;
  if (!std::isfinite(p.plane) || !std::isfinite(p.lat0) || !std::isfinite(p.lat1) || !std::isfinite(p.z0) ||
      !std::isfinite(p.z1))
    return false;
  for (uint32_t b = 0; b < nb; b++)
    if (!std::isfinite(p.trans[b])) return false;
  return true;
}

}  // namespace

extern "C" {

int32_t omg_dome_create(omg_ctx* ctx, uint32_t scene_id, const omg_dome_panel* glass, uint32_t n_glass,
                        uint32_t n_fan, uint32_t nb, uint32_t* probe_id) {
  if (!ctx || !probe_id || (n_glass && !glass) || n_fan == 0 || nb < 2 || nb > (uint32_t)MAXB) return OMG_E_INVALID;
  auto it = ctx->scenes.find(scene_id);
  if (it == ctx->scenes.end()) return OMG_E_NOT_FOUND;
  if (it->second->n_bands != nb) return OMG_E_INVALID;
  std::shared_ptr<DomeRec> D(new DomeRec());
  D->scene_id = scene_id;
  D->n_fan = n_fan;
  D->nb = nb;
  for (uint32_t i = 0; i < n_glass; i++) {
    if (!valid_dome_panel(glass[i], nb)) return OMG_E_INVALID;
    D->glass.push_back(to_dpanel(glass[i], nb));
  }
  CK(D->fan.alloc(n_fan));
  CK(build_dome_fan(D->fan.p, n_fan, ctx->stream));
  CK(D->hdr.alloc(1));
  CK(D->events.alloc(2));
  CK(cudaEventCreateWithFlags(&D->done, cudaEventDisableTiming));
  CK(cudaStreamSynchronize(ctx->stream));
  *probe_id = ctx->next_probe++;
  ctx->probes[*probe_id] = D;
  return OMG_OK;
}

int32_t omg_dome_destroy(omg_ctx* ctx, uint32_t probe_id) {
  if (!ctx) return OMG_E_INVALID;
  auto it = ctx->probes.find(probe_id);
  if (it == ctx->probes.end()) return OMG_E_NOT_FOUND;
  // a submitted sample may still use the probe's buffers (on any stream)
  if (it->second->pending) {
    int32_t rc = wait_event(ctx, it->second->done, timeout_of(ctx));
    if (rc) return rc;
  }
  cudaStreamSynchronize(ctx->stream);
  ctx->probes.erase(it);
  return OMG_OK;
}

}  // extern "C"

namespace {

enum : uint32_t { kWantRaw = 1, kWantEscape = 2, kWantTp = 4 };

// Enqueue one sample on stream s: inputs through pinned staging, the dome
// kernels, results into pinned staging, then the probe's event.
int32_t dome_submit(omg_ctx* ctx, DomeRec& D, const float* eyes, uint32_t n_eyes, const omg_dome_panel* leaves,
                    uint32_t n_leaves, uint32_t n_rays, uint32_t max_events, uint32_t flags, cudaStream_t s) {
  if (!eyes || !n_eyes || (n_leaves && !leaves) || n_rays == 0 || max_events == 0) return OMG_E_INVALID;
  if (n_rays > D.n_fan) return OMG_E_INVALID;
  if (D.pending) {
    ctx->last_error = "dome: the previous sample was not collected";
    return OMG_E_INVALID;
  }
  auto sit = ctx->scenes.find(D.scene_id);
  if (sit == ctx->scenes.end()) return OMG_E_NOT_FOUND;
  for (uint32_t i = 0; i < 3 * n_eyes; i++)
    if (!std::isfinite(eyes[i])) return OMG_E_INVALID;
  const uint32_t nb = D.nb;
  std::vector<DDomePanel> pans = D.glass;
  for (uint32_t i = 0; i < n_leaves; i++) {
    if (!valid_dome_panel(leaves[i], nb)) return OMG_E_INVALID;
    pans.push_back(to_dpanel(leaves[i], nb));
  }
  if (n_eyes > D.eye_cap) {
    // grow the per-listener EMA state, keeping existing slots
    uint32_t cap = std::max(n_eyes, D.eye_cap * 2);
    DevBuf<float> ema;
    DevBuf<uint32_t> primed;
    CK(ema.alloc((size_t)cap * 9 * nb));
    CK(primed.alloc(cap));
    CK(cudaMemsetAsync(ema.p, 0, (size_t)cap * 9 * nb * 4, s));
    CK(cudaMemsetAsync(primed.p, 0, (size_t)cap * 4, s));
    if (D.eye_cap) {
      CK(cudaMemcpyAsync(ema.p, D.ema.p, (size_t)D.eye_cap * 9 * nb * 4, cudaMemcpyDeviceToDevice, s));
      CK(cudaMemcpyAsync(primed.p, D.primed.p, (size_t)D.eye_cap * 4, cudaMemcpyDeviceToDevice, s));
    }
    CK(cudaStreamSynchronize(s));
    std::swap(D.ema.p, ema.p);
    std::swap(D.ema.n, ema.n);
    std::swap(D.primed.p, primed.p);
    std::swap(D.primed.n, primed.n);
    D.eye_cap = cap;
  }
  const uint64_t nr = (uint64_t)n_eyes * n_rays;
  if (D.eyes.n < 3ull * n_eyes) {
    CK(D.eyes.alloc(3ull * n_eyes));
    CK(D.h_eyes.alloc(3ull * n_eyes));
  }
  if (D.tp.n < nr * nb) CK(D.tp.alloc(nr * nb));
  if (D.esc.n < nr) CK(D.esc.alloc(nr));
  if (D.raw.n < 9ull * nb * n_eyes) {
    CK(D.raw.alloc(9ull * nb * n_eyes));
    CK(D.energy.alloc(9ull * nb * n_eyes));
    CK(D.dir.alloc(27ull * n_eyes));
    CK(D.h_raw.alloc(9ull * nb * n_eyes));
    CK(D.h_energy.alloc(9ull * nb * n_eyes));
    CK(D.h_dir.alloc(27ull * n_eyes));
  }
  if ((flags & kWantEscape) && D.h_esc.n < nr) CK(D.h_esc.alloc(nr));
  if ((flags & kWantTp) && D.h_tp.n < nr * nb) CK(D.h_tp.alloc(nr * nb));
  if (D.panels.n < pans.size()) {
    CK(D.panels.alloc(pans.size()));
    CK(D.h_panels.alloc(pans.size()));
  }
  if (!D.h_hdr.p) {
    CK(D.h_hdr.alloc(1));
    CK(D.h_events.alloc(2));
  }
  std::memcpy(D.h_eyes.p, eyes, 12ull * n_eyes);
  CK(cudaMemcpyAsync(D.eyes.p, D.h_eyes.p, 12ull * n_eyes, cudaMemcpyHostToDevice, s));
  if (!pans.empty()) {
    std::memcpy(D.h_panels.p, pans.data(), pans.size() * sizeof(DDomePanel));
    CK(cudaMemcpyAsync(D.panels.p, D.h_panels.p, pans.size() * sizeof(DDomePanel), cudaMemcpyHostToDevice, s));
  }
  CK(cudaMemsetAsync(D.hdr.p, 0, sizeof(DLaunch), s));
  CK(cudaMemsetAsync(D.events.p, 0, 8, s));
  DDomeLaunch L;
  std::memset(&L, 0, sizeof(L));
  L.scene = ctx->d_scenes.p + D.scene_id;
  L.fan = D.fan.p;
  L.n_fan = D.n_fan;
  L.n_rays = n_rays;
  L.max_events = max_events;
  L.nb = nb;
  L.panels = D.panels.p;
  L.n_glass = (uint32_t)D.glass.size();
  L.n_panels = (uint32_t)pans.size();
  L.eyes = D.eyes.p;
  L.n_eyes = n_eyes;
  L.ray_tp = D.tp.p;
  L.ray_escape = D.esc.p;
  L.ema = D.ema.p;
  L.primed = D.primed.p;
  L.raw = D.raw.p;
  L.out_dir = D.dir.p;
  L.out_energy = D.energy.p;
  L.hdr = D.hdr.p;
  L.events = D.events.p;
  L.tie = ctx->prm.tie_mode;
  L.wt = ctx->prm.tri_test == OMG_TRI_WATERTIGHT ? 1u : 0u;
  CK(launch_dome(L, s));
  CK(cudaMemcpyAsync(D.h_energy.p, D.energy.p, 9ull * nb * n_eyes * 4, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(D.h_dir.p, D.dir.p, 27ull * n_eyes * 4, cudaMemcpyDeviceToHost, s));
  if (flags & kWantRaw) CK(cudaMemcpyAsync(D.h_raw.p, D.raw.p, 9ull * nb * n_eyes * 4, cudaMemcpyDeviceToHost, s));
  if (flags & kWantEscape) CK(cudaMemcpyAsync(D.h_esc.p, D.esc.p, nr, cudaMemcpyDeviceToHost, s));
  if (flags & kWantTp) CK(cudaMemcpyAsync(D.h_tp.p, D.tp.p, nr * nb * 4, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(D.h_hdr.p, D.hdr.p, sizeof(DLaunch), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(D.h_events.p, D.events.p, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaEventRecord(D.done, s));
  D.pending = true;
  D.p_eyes = n_eyes;
  D.p_rays = n_rays;
  D.p_flags = flags;
  return OMG_OK;
}

// Wait (bounded) for a submitted sample and copy its results out.
int32_t dome_collect(omg_ctx* ctx, DomeRec& D, omg_dome_bin* out, float* raw_energy, uint8_t* escape,
                     float* ray_tp) {
  if (!D.pending) {
    ctx->last_error = "dome: nothing submitted";
    return OMG_E_INVALID;
  }
  int32_t rc = wait_event(ctx, D.done, timeout_of(ctx));
  if (rc) return rc;
  D.pending = false;
  const uint32_t nb = D.nb, n_eyes = D.p_eyes;
  const uint64_t nr = (uint64_t)n_eyes * D.p_rays;
  ctx->last_flags = D.h_hdr.p->error;
  if (D.h_hdr.p->error) {
    ctx->last_error = (D.h_hdr.p->error & 2u) ? "dome: too many crossings on one straight-through segment"
                                              : "dome: traversal stack overflow";
    return OMG_E_OVERFLOW;
  }
  D.last_events[0] = D.h_events.p[0];
  D.last_events[1] = D.h_events.p[1];
  if (out)
    for (uint32_t e = 0; e < n_eyes; e++)
      for (uint32_t k = 0; k < 9; k++) {
        omg_dome_bin& o = out[e * 9 + k];
        std::memset(&o, 0, sizeof(o));
        for (int c = 0; c < 3; c++) o.dir[c] = D.h_dir.p[(e * 9 + k) * 3 + c];
        for (uint32_t b = 0; b < nb; b++) o.energy[b] = D.h_energy.p[(e * 9 + k) * nb + b];
      }
  if (raw_energy && (D.p_flags & kWantRaw)) std::memcpy(raw_energy, D.h_raw.p, 9ull * nb * n_eyes * 4);
  if (escape && (D.p_flags & kWantEscape)) std::memcpy(escape, D.h_esc.p, nr);
  if (ray_tp && (D.p_flags & kWantTp)) std::memcpy(ray_tp, D.h_tp.p, nr * nb * 4);
  return OMG_OK;
}

}  // namespace

extern "C" {

int32_t omg_dome_sample(omg_ctx* ctx, uint32_t probe_id, const float* eyes, uint32_t n_eyes,
                        const omg_dome_panel* leaves, uint32_t n_leaves, uint32_t n_rays, uint32_t max_events,
                        omg_dome_bin* out, float* raw_energy, uint8_t* escape, float* ray_tp) {
  if (!ctx || !out) return OMG_E_INVALID;
  auto it = ctx->probes.find(probe_id);
  if (it == ctx->probes.end()) return OMG_E_NOT_FOUND;
  DomeRec& D = *it->second;
  const uint32_t flags = (raw_energy ? kWantRaw : 0u) | (escape ? kWantEscape : 0u) | (ray_tp ? kWantTp : 0u);
  int32_t rc = dome_submit(ctx, D, eyes, n_eyes, leaves, n_leaves, n_rays, max_events, flags, ctx->stream);
  if (rc) return rc;
  return dome_collect(ctx, D, out, raw_energy, escape, ray_tp);
}

int32_t omg_dome_submit(omg_ctx* ctx, uint32_t probe_id, const float* eyes, uint32_t n_eyes,
                        const omg_dome_panel* leaves, uint32_t n_leaves, uint32_t n_rays, uint32_t max_events,
                        uint32_t want, void* cuda_stream) {
  if (!ctx) return OMG_E_INVALID;
  auto it = ctx->probes.find(probe_id);
  if (it == ctx->probes.end()) return OMG_E_NOT_FOUND;
  cudaStream_t s = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : ctx->stream;
  return dome_submit(ctx, *it->second, eyes, n_eyes, leaves, n_leaves, n_rays, max_events, want & 7u, s);
}

int32_t omg_dome_collect(omg_ctx* ctx, uint32_t probe_id, omg_dome_bin* out, float* raw_energy, uint8_t* escape,
                         float* ray_tp) {
  if (!ctx) return OMG_E_INVALID;
  auto it = ctx->probes.find(probe_id);
  if (it == ctx->probes.end()) return OMG_E_NOT_FOUND;
  return dome_collect(ctx, *it->second, out, raw_energy, escape, ray_tp);
}

// Segments (escape events + straight-through calls) of the probe's last sample.
int32_t omg_dome_segments(omg_ctx* ctx, uint32_t probe_id, uint64_t* escape_events, uint64_t* through_calls) {
  if (!ctx) return OMG_E_INVALID;
  auto it = ctx->probes.find(probe_id);
  if (it == ctx->probes.end()) return OMG_E_NOT_FOUND;
  if (escape_events) *escape_events = it->second->last_events[0];
  if (through_calls) *through_calls = it->second->last_events[1];
  return OMG_OK;
}

}  // extern "C"
