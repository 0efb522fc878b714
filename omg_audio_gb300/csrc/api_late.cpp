// C ABI of the GB300 tracer (include/omg_cuda.h), part 5: the late field of
// many sim instances (Sim::reverb_world / reverb_only, crates/omg-scene/src/
// sim.rs:330-398) with device-resident averaged echograms.
#include "runtime.h"

using namespace omg;

namespace omg {

struct LateRec {
  uint32_t n_slots = 0, n_bins = 0, nb = 0, from_bin = 0;
  float bin_dt = 0.0f;
  DevBuf<float> avg;               // n_slots x n_bins x (nb + 3): bins then dirs per slot
  DevBuf<uint32_t> version;        // updates per slot
  DevBuf<omg_late_state> state;    // n_slots
  DevBuf<DLateUpdate> d_up;        // the tick's updates (<= n_slots)
  DevBuf<DReverbJob> d_rj;
  DevBuf<omg_reverb> d_rev;
  PinBuf<DLateUpdate> h_up;
  PinBuf<DReverbJob> h_rj;
  PinBuf<omg_late_state> h_state;
  // batch records of recent job layouts (the number of traced slots varies by tick)
  std::vector<std::unique_ptr<BatchRec>> cache;
  BatchRec* inflight = nullptr;
  cudaEvent_t done = nullptr;
  bool pending = false;
  uint32_t tick = 0, done_tick = 0;
  std::vector<uint32_t> updates;   // updates submitted per slot (the default weight)
  ~LateRec() {
    if (done) cudaEventDestroy(done);
  }
};

}  // namespace omg

namespace {

constexpr size_t kLateCache = 4;

// Wait (bounded) for the tick in flight, if any, and settle its status.
int32_t late_settle(omg_ctx* ctx, LateRec& L) {
  if (!L.pending) return OMG_OK;
  int32_t rc = wait_event(ctx, L.done, timeout_of(ctx));
  if (rc) return rc;
  L.pending = false;
  L.done_tick = L.tick;
  if (L.inflight) return batch_flags(ctx, *L.inflight);
  return OMG_OK;
}

// The state of a slot that was never traced: estimate_reverb and
// late_direction of an empty echogram (tracer.rs:70-72, 213-256).
omg_late_state empty_state() {
  omg_late_state s;
  std::memset(&s, 0, sizeof(s));
  for (int b = 0; b < OMG_MAX_BANDS; b++) s.rt60[b] = 0.5f;
  s.dir[0] = 1.0f;
  return s;
}

LateRec* find_late(omg_ctx* ctx, uint32_t id) {
  auto it = ctx->lates.find(id);
  return it == ctx->lates.end() ? nullptr : it->second.get();
}

}  // namespace

extern "C" {

int32_t omg_late_create(omg_ctx* ctx, uint32_t n_slots, float dir_from_s, uint32_t* field_id) {
  if (!ctx || !field_id || n_slots == 0 || n_slots > (1u << 20) || !(dir_from_s >= 0.0f)) return OMG_E_INVALID;
  const omg_params& P = ctx->prm;
  std::shared_ptr<LateRec> L(new LateRec());
  L->n_slots = n_slots;
  L->updates.assign(n_slots, 0);
  L->n_bins = P.n_bins;
  L->nb = P.n_bands;
  L->bin_dt = P.bin_dt;
  // tracer.rs:60: (from_s / BIN_DT) as usize, in f32
  const float q = dir_from_s / P.bin_dt;
  L->from_bin = q >= (float)P.n_bins ? P.n_bins : (uint32_t)q;
  const uint64_t per = (uint64_t)L->n_bins * (L->nb + 3);
  CK(L->avg.alloc(per * n_slots));
  CK(L->version.alloc(n_slots));
  CK(L->state.alloc(n_slots));
  CK(L->d_up.alloc(n_slots));
  CK(L->d_rj.alloc(n_slots));
  CK(L->d_rev.alloc(n_slots));
  CK(L->h_up.alloc(n_slots));
  CK(L->h_rj.alloc(n_slots));
  CK(L->h_state.alloc(n_slots));
  CK(cudaMemsetAsync(L->avg.p, 0, per * n_slots * sizeof(float), ctx->stream));
  CK(cudaMemsetAsync(L->version.p, 0, n_slots * sizeof(uint32_t), ctx->stream));
  for (uint32_t i = 0; i < n_slots; i++) L->h_state.p[i] = empty_state();
  CK(cudaMemcpyAsync(L->state.p, L->h_state.p, n_slots * sizeof(omg_late_state), cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(cudaEventCreateWithFlags(&L->done, cudaEventDisableTiming));
  CK(cudaStreamSynchronize(ctx->stream));
  *field_id = ctx->next_late++;
  ctx->lates[*field_id] = L;
  return OMG_OK;
}

int32_t omg_late_destroy(omg_ctx* ctx, uint32_t field_id) {
  if (!ctx) return OMG_E_INVALID;
  LateRec* L = find_late(ctx, field_id);
  if (!L) return OMG_E_NOT_FOUND;
  int32_t rc = late_settle(ctx, *L);
  ctx->lates.erase(field_id);
  return rc == OMG_E_OVERFLOW ? OMG_OK : rc;
}

int32_t omg_late_submit(omg_ctx* ctx, uint32_t field_id, const uint32_t* slots, const omg_job* jobs,
                        const float* alpha, uint32_t n_jobs, const omg_panel* panels, uint32_t n_panels,
                        uint32_t* tick) {
  if (!ctx || !tick || (n_jobs && (!slots || !jobs)) || (n_panels && !panels)) return OMG_E_INVALID;
  LateRec* Lp = find_late(ctx, field_id);
  if (!Lp) return OMG_E_NOT_FOUND;
  LateRec& L = *Lp;
  if (L.pending) return OMG_PENDING;
  if (n_jobs > L.n_slots) return OMG_E_INVALID;
  std::vector<uint8_t> seen(L.n_slots, 0);
  for (uint32_t i = 0; i < n_jobs; i++) {
    const uint32_t nb = jobs[i].n_bands ? jobs[i].n_bands : ctx->prm.n_bands;
    const uint32_t n_bins = jobs[i].n_bins ? jobs[i].n_bins : ctx->prm.n_bins;
    if (slots[i] >= L.n_slots || seen[slots[i]] || nb != L.nb || n_bins != L.n_bins) return OMG_E_INVALID;
    if (alpha && !(alpha[i] >= 0.0f && alpha[i] <= 1.0f)) return OMG_E_INVALID;
    seen[slots[i]] = 1;
  }
  BatchRec* B = nullptr;
  if (n_jobs) {
    const uint64_t sig = batch_layout(jobs, n_jobs, n_panels, ctx->prm);
    size_t hit = L.cache.size();
    for (size_t k = 0; k < L.cache.size(); k++)
      if (L.cache[k]->signature == sig) hit = k;
    int32_t rc = OMG_OK;
    if (hit < L.cache.size()) {
      // most recently used last
      std::unique_ptr<BatchRec> b = std::move(L.cache[hit]);
      L.cache.erase(L.cache.begin() + (ptrdiff_t)hit);
      L.cache.push_back(std::move(b));
      rc = batch_refill(ctx, *L.cache.back(), jobs, n_jobs, panels, n_panels);
    } else {
      if (L.cache.size() >= kLateCache) L.cache.erase(L.cache.begin());
      L.cache.emplace_back(new BatchRec());
      rc = batch_prepare(ctx, *L.cache.back(), jobs, n_jobs, panels, n_panels);
      if (rc) L.cache.pop_back();
    }
    if (rc) return rc;
    B = L.cache.back().get();
    const uint64_t per = (uint64_t)L.n_bins * (L.nb + 3);
    for (uint32_t i = 0; i < n_jobs; i++) {
      const float a = alpha ? alpha[i] : (L.updates[slots[i]] == 0 ? 1.0f : 0.3f);
      L.updates[slots[i]]++;
      L.h_up.p[i] = DLateUpdate{slots[i], L.tick + 1, B->jobs[i].out_off, a, 0};
      L.h_rj.p[i] = DReverbJob{(uint64_t)slots[i] * per, L.n_bins, L.nb, L.bin_dt, 0};
    }
    std::memcpy(B->h_jobs.p, B->jobs.data(), n_jobs * sizeof(DJob));
    CK(cudaMemcpyAsync(B->d_jobs.p, B->h_jobs.p, n_jobs * sizeof(DJob), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaGraphLaunch(B->graph, ctx->stream));
    CK(cudaMemcpyAsync(L.d_up.p, L.h_up.p, n_jobs * sizeof(DLateUpdate), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(L.d_rj.p, L.h_rj.p, n_jobs * sizeof(DReverbJob), cudaMemcpyHostToDevice, ctx->stream));
    CK(launch_late_update(L.d_up.p, n_jobs, B->d_out.p, L.avg.p, L.version.p, L.d_rj.p, L.d_rev.p, L.state.p,
                          L.n_bins, L.nb, L.from_bin, ctx->prm.dir_band, ctx->stream));
    CK(cudaMemcpyAsync(B->h_hdr.p, B->d_hdr.p, sizeof(DLaunch), cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaMemcpyAsync(L.h_state.p, L.state.p, L.n_slots * sizeof(omg_late_state), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaEventRecord(L.done, ctx->stream));
  L.inflight = B;
  L.pending = true;
  *tick = ++L.tick;
  return OMG_OK;
}

int32_t omg_late_poll(omg_ctx* ctx, uint32_t field_id, omg_late_state* states, uint32_t* tick) {
  if (!ctx || !states) return OMG_E_INVALID;
  LateRec* Lp = find_late(ctx, field_id);
  if (!Lp) return OMG_E_NOT_FOUND;
  LateRec& L = *Lp;
  if (L.pending) {
    cudaError_t q = cudaEventQuery(L.done);
    if (q == cudaErrorNotReady) return OMG_PENDING;
    if (q != cudaSuccess) return fail(ctx, q, "cudaEventQuery");
    L.pending = false;
    L.done_tick = L.tick;
    if (L.inflight) {
      int32_t rc = batch_flags(ctx, *L.inflight);
      if (rc) return rc;
    }
  }
  std::memcpy(states, L.h_state.p, L.n_slots * sizeof(omg_late_state));
  if (tick) *tick = L.done_tick;
  return OMG_OK;
}

int32_t omg_late_reset(omg_ctx* ctx, uint32_t field_id, uint32_t slot) {
  if (!ctx) return OMG_E_INVALID;
  LateRec* Lp = find_late(ctx, field_id);
  if (!Lp) return OMG_E_NOT_FOUND;
  LateRec& L = *Lp;
  if (L.pending) return OMG_PENDING;
  if (slot >= L.n_slots) return OMG_E_INVALID;
  const uint64_t per = (uint64_t)L.n_bins * (L.nb + 3);
  CK(cudaMemsetAsync(L.avg.p + per * slot, 0, per * sizeof(float), ctx->stream));
  CK(cudaMemsetAsync(L.version.p + slot, 0, sizeof(uint32_t), ctx->stream));
  L.h_state.p[slot] = empty_state();
  CK(cudaMemcpyAsync(L.state.p + slot, L.h_state.p + slot, sizeof(omg_late_state), cudaMemcpyHostToDevice,
                     ctx->stream));
  L.updates[slot] = 0;
  CK(cudaStreamSynchronize(ctx->stream));
  return OMG_OK;
}

int32_t omg_late_read(omg_ctx* ctx, uint32_t field_id, uint32_t slot, float* bins, float* dirs) {
  if (!ctx) return OMG_E_INVALID;
  LateRec* Lp = find_late(ctx, field_id);
  if (!Lp) return OMG_E_NOT_FOUND;
  LateRec& L = *Lp;
  if (L.pending) return OMG_PENDING;
  if (slot >= L.n_slots) return OMG_E_INVALID;
  const uint64_t per = (uint64_t)L.n_bins * (L.nb + 3), nbb = (uint64_t)L.n_bins * L.nb;
  if (bins) CK(cudaMemcpy(bins, L.avg.p + per * slot, nbb * sizeof(float), cudaMemcpyDeviceToHost));
  if (dirs) CK(cudaMemcpy(dirs, L.avg.p + per * slot + nbb, (uint64_t)L.n_bins * 3 * sizeof(float),
                          cudaMemcpyDeviceToHost));
  return OMG_OK;
}

}  // extern "C"
