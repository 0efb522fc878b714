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
  cudaStreamSynchronize(ctx->stream);
  ctx->probes.erase(it);
  return OMG_OK;
}

int32_t omg_dome_sample(omg_ctx* ctx, uint32_t probe_id, const float* eyes, uint32_t n_eyes,
                        const omg_dome_panel* leaves, uint32_t n_leaves, uint32_t n_rays, uint32_t max_events,
                        omg_dome_bin* out, float* raw_energy, uint8_t* escape, float* ray_tp) {
  if (!ctx || !eyes || !n_eyes || (n_leaves && !leaves) || !out || n_rays == 0 || max_events == 0)
    return OMG_E_INVALID;
  auto it = ctx->probes.find(probe_id);
  if (it == ctx->probes.end()) return OMG_E_NOT_FOUND;
  DomeRec& D = *it->second;
  if (n_rays > D.n_fan) return OMG_E_INVALID;
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
  cudaStream_t s = ctx->stream;
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
  if (D.eyes.n < 3ull * n_eyes) CK(D.eyes.alloc(3ull * n_eyes));
  if (D.tp.n < nr * nb) CK(D.tp.alloc(nr * nb));
  if (D.esc.n < nr) CK(D.esc.alloc(nr));
  if (D.raw.n < 9ull * nb * n_eyes) {
    CK(D.raw.alloc(9ull * nb * n_eyes));
    CK(D.energy.alloc(9ull * nb * n_eyes));
    CK(D.dir.alloc(27ull * n_eyes));
  }
  if (D.panels.n < pans.size()) CK(D.panels.alloc(pans.size()));
  CK(cudaMemcpyAsync(D.eyes.p, eyes, 12ull * n_eyes, cudaMemcpyHostToDevice, s));
  if (!pans.empty())
    CK(cudaMemcpyAsync(D.panels.p, pans.data(), pans.size() * sizeof(DDomePanel), cudaMemcpyHostToDevice, s));
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
  CK(launch_dome(L, s));
  std::vector<float> energy(9ull * nb * n_eyes), dir(27ull * n_eyes);
  CK(cudaMemcpyAsync(energy.data(), D.energy.p, energy.size() * 4, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(dir.data(), D.dir.p, dir.size() * 4, cudaMemcpyDeviceToHost, s));
  if (raw_energy) CK(cudaMemcpyAsync(raw_energy, D.raw.p, 9ull * nb * n_eyes * 4, cudaMemcpyDeviceToHost, s));
  if (escape) CK(cudaMemcpyAsync(escape, D.esc.p, nr, cudaMemcpyDeviceToHost, s));
  if (ray_tp) CK(cudaMemcpyAsync(ray_tp, D.tp.p, nr * nb * 4, cudaMemcpyDeviceToHost, s));
  DLaunch h;
  uint32_t ev[2];
  CK(cudaMemcpyAsync(&h, D.hdr.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(ev, D.events.p, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaEventRecord(D.done, s));
  int32_t rc = wait_event(ctx, D.done, timeout_of(ctx));
  if (rc) return rc;
  if (h.error) {
    ctx->last_error = (h.error & 2u) ? "dome: too many crossings on one straight-through segment"
                                     : "dome: traversal stack overflow";
    return OMG_E_OVERFLOW;
  }
  D.last_events[0] = ev[0];
  D.last_events[1] = ev[1];
  for (uint32_t e = 0; e < n_eyes; e++)
    for (uint32_t k = 0; k < 9; k++) {
      omg_dome_bin& o = out[e * 9 + k];
      std::memset(&o, 0, sizeof(o));
      for (int c = 0; c < 3; c++) o.dir[c] = dir[(e * 9 + k) * 3 + c];
      for (uint32_t b = 0; b < nb; b++) o.energy[b] = energy[(e * 9 + k) * nb + b];
    }
  return OMG_OK;
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
