// C ABI of the GB300 tracer (include/omg_cuda.h), part 1: contexts, batches,
// CUDA-graph launches, bounded waits, async tickets, the autotuner.
#include "runtime.h"

using namespace omg;

namespace omg {

int32_t fail(omg_ctx* ctx, cudaError_t e, const char* where) {
  char buf[256];
  std::snprintf(buf, sizeof(buf), "%s: %s", where, cudaGetErrorString(e));
  ctx->last_error = buf;
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? OMG_E_OOM : OMG_E_DEVICE;
}

uint32_t timeout_of(const omg_ctx* ctx) { return ctx->prm.timeout_ms ? ctx->prm.timeout_ms : 10000u; }

// Bounded wait on an event: poll, never block indefinitely.
int32_t wait_event(omg_ctx* ctx, cudaEvent_t ev, uint32_t timeout_ms) {
  auto t0 = std::chrono::steady_clock::now();
  while (true) {
    cudaError_t q = cudaEventQuery(ev);
    if (q == cudaSuccess) return OMG_OK;
    if (q != cudaErrorNotReady) return fail(ctx, q, "cudaEventQuery");
    auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
    if ((uint64_t)ms >= timeout_ms) {
      ctx->last_error = "timeout waiting for the device";
      return OMG_E_TIMEOUT;
    }
    // a yielding spin: the calling thread waits for this result anyway, and a
    // timed sleep would wake up tens of microseconds after the event
    std::this_thread::yield();
  }
}

bool valid_material(const omg_material& m, uint32_t nb) {
  for (uint32_t b = 0; b < nb; b++) {
    if (!std::isfinite(m.absorption[b]) || !std::isfinite(m.transmission[b])) return false;
  }
  return std::isfinite(m.scattering);
}

bool finite3(const float* v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

// walk_cap: omg_params.walk_budget (0: no cap below the structural bound)
DScene scene_view(const SceneRec& s, uint32_t walk_cap) {
  DScene d;
  std::memset(&d, 0, sizeof(d));
  d.nodes = s.nodes.p;
  d.prims = s.prims.p;
  d.normals = s.normals.p;
  d.mats = s.mats.p;
  d.tri_surface = s.tri_surface.p;
  d.root = s.root;
  d.n_nodes = s.n_nodes;
  d.n_prims = s.n_prims;
  d.n_bands = s.n_bands;
  d.nodes4 = s.n_nodes4 ? s.nodes4.p : nullptr;
  d.nodes4c = s.n_nodes4 ? s.nodes4c.p : nullptr;
  d.nodes_f = s.nodes_f.p;
  d.prims_wt = s.prims_wt.p;
  for (int a = 0; a < 3; a++) d.fast_m[a] = s.fast_m[a];
  d.root4 = s.root4;
  d.n_nodes4 = s.n_nodes4;
  const uint64_t b2 = 2ull * s.n_nodes + s.n_prims + 64ull, b4 = (uint64_t)s.n_nodes4 + 1ull;
  const uint64_t cap = walk_cap ? walk_cap : 0xFFFFFFFFull;
  d.walk_budget = (uint32_t)std::min(std::min(b2, cap), (uint64_t)0xFFFFFFFFull);
  d.walk_budget4 = (uint32_t)std::min(b4, cap);
  return d;
}

// The device scene table has a fixed capacity for the context's lifetime:
// captured graphs hold its address, so it is never reallocated.
int32_t sync_scene_table(omg_ctx* ctx) {
  if (ctx->scene_cap == 0) {
    CK(ctx->d_scenes.alloc(kMaxScenes));
    CK(cudaMemset(ctx->d_scenes.p, 0, kMaxScenes * sizeof(DScene)));
    ctx->scene_cap = kMaxScenes;
  }
  std::vector<DScene> table(ctx->scene_cap);
  std::memset(table.data(), 0, table.size() * sizeof(DScene));
  for (auto& kv : ctx->scenes) table[kv.first] = scene_view(*kv.second, ctx->prm.walk_budget);
  CK(cudaMemcpy(ctx->d_scenes.p, table.data(), table.size() * sizeof(DScene), cudaMemcpyHostToDevice));
  return OMG_OK;
}

}  // namespace omg

namespace {

// ---------------------------------------------------------------- batches
uint64_t batch_signature(const omg_job* jobs, uint32_t n, uint32_t n_panels, const omg_params& P) {
  uint64_t h = 1469598103934665603ULL ^ n ^ ((uint64_t)n_panels << 32);
  auto mix = [&](uint64_t v) { h = (h ^ v) * 1099511628211ULL; };
  for (uint32_t i = 0; i < n; i++) {
    const omg_job& j = jobs[i];
    mix(j.geom);
    mix(j.scene_id);
    mix(j.n_rays);
    mix(j.n_bands ? j.n_bands : P.n_bands);
    mix(j.n_bins ? j.n_bins : P.n_bins);
    mix(j.n_panels);
    mix(j.panel_offset);
  }
  return h;
}

// Sort a job's panels along a Morton curve of their centres and group them by
// 4 behind union boxes (the trace kernel skips a group whose box misses the
// segment). Panel order only matters for exact ties, which the kernel settles
// by the original index.
void group_panels(std::vector<DPanel>& jp, uint32_t base, std::vector<DPanelGroup>& groups, uint32_t& group_off,
                  uint32_t& n_groups) {
  group_off = (uint32_t)groups.size();
  n_groups = 0;
  if (jp.empty()) return;
  float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
  for (const DPanel& p : jp)
    for (int c = 0; c < 3; c++) {
      lo[c] = std::min(lo[c], 0.5f * (p.mn[c] + p.mx[c]));
      hi[c] = std::max(hi[c], 0.5f * (p.mn[c] + p.mx[c]));
    }
  auto spread = [](uint32_t v) {
    uint64_t x = v & 0x1FFFFF;
    x = (x | x << 32) & 0x1F00000000FFFFull;
    x = (x | x << 16) & 0x1F0000FF0000FFull;
    x = (x | x << 8) & 0x100F00F00F00F00Full;
    x = (x | x << 4) & 0x10C30C30C30C30C3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
  };
  std::vector<std::pair<uint64_t, uint32_t>> key(jp.size());
  for (size_t i = 0; i < jp.size(); i++) {
    uint32_t q[3];
    for (int c = 0; c < 3; c++) {
      float e = hi[c] - lo[c];
      float u = e > 0 ? (0.5f * (jp[i].mn[c] + jp[i].mx[c]) - lo[c]) / e : 0.0f;
      q[c] = (uint32_t)std::min(std::max(u * 1048575.0f, 0.0f), 1048575.0f);
    }
    key[i] = {(spread(q[0]) << 2) | (spread(q[1]) << 1) | spread(q[2]), (uint32_t)i};
  }
  std::stable_sort(key.begin(), key.end());
  std::vector<DPanel> sorted(jp.size());
  for (size_t i = 0; i < jp.size(); i++) sorted[i] = jp[key[i].second];
  jp.swap(sorted);
  for (size_t g = 0; g < jp.size(); g += 4) {
    DPanelGroup G;
    std::memset(&G, 0, sizeof(G));
    G.first = base + (uint32_t)g;
    G.count = (uint32_t)std::min<size_t>(4, jp.size() - g);
    for (int c = 0; c < 3; c++) {
      G.mn[c] = jp[g].mn[c];
      G.mx[c] = jp[g].mx[c];
    }
    for (uint32_t k = 1; k < G.count; k++)
      for (int c = 0; c < 3; c++) {
        G.mn[c] = std::min(G.mn[c], jp[g + k].mn[c]);
        G.mx[c] = std::max(G.mx[c], jp[g + k].mx[c]);
      }
    groups.push_back(G);
    n_groups++;
  }
}

// Fill the host-side job arrays of a batch (no device work).
int32_t fill_batch(omg_ctx* ctx, BatchRec& B, const omg_job* jobs, uint32_t n_jobs, const omg_panel* panels,
                   uint32_t n_panels) {
  const omg_params& P = ctx->prm;
  B.n_jobs = n_jobs;
  B.jobs.assign(n_jobs, DJob{});
  B.job_mats.clear();
  B.panels.clear();
  B.groups.clear();
  B.rjobs.assign(n_jobs, DReverbJob{});
  uint64_t acc = 0, out = 0, rays = 0;
  B.max_nb = 0;
  B.max_bins = 0;
  B.n_bin_floats = 0;
  B.n_dir_floats = 0;
  bool coop_ok = P.tie_mode != 0;
  // per-job panel materials are placed after all box wall materials
  for (uint32_t i = 0; i < n_jobs; i++) {
    const omg_job& j = jobs[i];
    DJob& d = B.jobs[i];
    std::memset(&d, 0, sizeof(d));
    uint32_t nb = j.n_bands ? j.n_bands : P.n_bands;
    uint32_t n_bins = j.n_bins ? j.n_bins : P.n_bins;
    float max_time = j.max_time > 0.0f ? j.max_time : P.max_time;
    if (nb == 0 || nb > (uint32_t)MAXB || n_bins == 0 || n_bins > kMaxBins || j.n_rays == 0) return OMG_E_INVALID;
    if (P.dir_band >= nb) return OMG_E_INVALID;
    if (!finite3(j.src) || !finite3(j.lis)) return OMG_E_INVALID;
    if ((uint64_t)j.panel_offset + j.n_panels > n_panels) return OMG_E_INVALID;
    d.geom = j.geom;
    d.n_rays = j.n_rays;
    d.seed = j.seed;
    for (int k = 0; k < 3; k++) {
      d.src[k] = j.src[k];
      d.lis[k] = j.lis[k];
    }
    d.per_ray = 1.0f / (float)j.n_rays;                     // tracer.rs:90
    d.floor_e = P.energy_floor * d.per_ray;                 // tracer.rs:163
    for (uint32_t b = 0; b < nb; b++) d.e0[b] = d.per_ray * j.energy[b];  // tracer.rs:95
    d.nb = nb;
    d.n_bins = n_bins;
    d.max_bounces = P.max_bounces;
    d.dir_band = P.dir_band;
    d.bin_dt = P.bin_dt;
    d.max_time = max_time;
    d.rr = P.receiver_radius;
    d.wall_eps = P.wall_eps;
    d.c = P.speed_of_sound;
    if (j.geom == OMG_GEOM_BOX) {
      if (!finite3(j.box_size)) return OMG_E_INVALID;
      for (int k = 0; k < 3; k++) d.box[k] = j.box_size[k];
      d.box_mat = (uint32_t)B.job_mats.size();
      for (int w = 0; w < 6; w++) {
        if (!valid_material(j.box_walls[w], nb)) return OMG_E_INVALID;
        B.job_mats.push_back(make_dmat(j.box_walls[w], nb));
      }
    } else if (j.geom == OMG_GEOM_MESH) {
      auto it = ctx->scenes.find(j.scene_id);
      if (it == ctx->scenes.end()) return OMG_E_NOT_FOUND;
      if (it->second->n_bands != nb) return OMG_E_INVALID;
      d.scene = j.scene_id;
      if (it->second->n_nodes4 == 0) coop_ok = false;
    } else {
      return OMG_E_INVALID;
    }
    d.panel_off = (uint32_t)B.panels.size();
    d.n_panels = j.n_panels;
    std::vector<DPanel> jp;
    for (uint32_t k = 0; k < j.n_panels; k++) {
      const omg_panel& p = panels[j.panel_offset + k];
      if (!finite3(p.mn) || !finite3(p.mx) || !valid_material(p.material, nb)) return OMG_E_INVALID;
      DPanel dp;
      std::memset(&dp, 0, sizeof(dp));
      for (int c = 0; c < 3; c++) {
        dp.mn[c] = p.mn[c];
        dp.mx[c] = p.mx[c];
      }
      dp.mat = (uint32_t)B.job_mats.size();
      dp.orig = k;
      B.job_mats.push_back(make_dmat(p.material, nb));
      jp.push_back(dp);
    }
    group_panels(jp, (uint32_t)B.panels.size(), B.groups, d.group_off, d.n_groups);
    B.panels.insert(B.panels.end(), jp.begin(), jp.end());
    d.ray_base = (uint32_t)rays;
    rays += j.n_rays;
    if (rays > 0xFFFFFFFFull) return OMG_E_INVALID;
    d.acc_off = acc;
    d.out_off = out;
    acc += acc_floats(n_bins, nb);
    out += out_floats(n_bins, nb);
    B.max_nb = std::max(B.max_nb, nb);
    B.max_bins = std::max(B.max_bins, n_bins);
    B.n_bin_floats += (uint64_t)n_bins * nb;
    B.n_dir_floats += (uint64_t)n_bins * 3;
    DReverbJob& r = B.rjobs[i];
    r.bins_off = d.out_off;
    r.n_bins = n_bins;
    r.nb = nb;
    r.bin_dt = P.bin_dt;
  }
  B.total_rays = (uint32_t)rays;
  B.coop_ok = coop_ok;
  B.n_acc = acc;
  B.n_out = out;
  return OMG_OK;
}

int32_t alloc_batch(omg_ctx* ctx, BatchRec& B) {
  CK(B.d_jobs.alloc(B.n_jobs));
  CK(B.d_job_mats.alloc(B.job_mats.size()));
  CK(B.d_panels.alloc(B.panels.size()));
  CK(B.d_groups.alloc(B.groups.size()));
  CK(B.d_acc.alloc(B.n_acc));
  CK(B.d_out.alloc(B.n_out));
  CK(B.d_hdr.alloc(1));
  CK(B.d_seg.alloc(B.n_jobs));
  CK(B.d_rjobs.alloc(B.n_jobs));
  CK(B.d_reverb.alloc(B.n_jobs));
  CK(B.h_out.alloc(B.n_out));
  CK(B.h_reverb.alloc(B.n_jobs));
  CK(B.h_hdr.alloc(1));
  CK(B.h_seg.alloc(B.n_jobs));
  CK(B.h_jobs.alloc(B.n_jobs));
  const size_t cap = B.total_rays;
  CK(B.d_wf_pos.alloc(cap));
  CK(B.d_wf_dir.alloc(cap));
  CK(B.d_wf_e.alloc(B.max_nb > 4 ? 2 * cap : cap));
  CK(B.d_wf_bounce.alloc(cap));
  CK(B.d_wf_queue.alloc(2 * cap));
  CK(B.d_wf_hit.alloc(cap));
  CK(B.d_wf_ctl.alloc(1));
  CK(B.d_ep_q.alloc(2 * cap));
  CK(B.d_ep_ctl.alloc(kMaxEpochs + 1));
  B.wf = WfState{B.d_wf_pos.p, B.d_wf_dir.p, B.d_wf_e.p, B.d_wf_bounce.p, B.d_wf_hit.p, B.d_wf_queue.p,
                 B.d_wf_ctl.p, B.total_rays};
  if (!B.done) CK(cudaEventCreateWithFlags(&B.done, cudaEventDisableTiming));
  return OMG_OK;
}

// Upload the job-dependent arrays (synchronous on the context stream).
int32_t upload_batch(omg_ctx* ctx, BatchRec& B) {
  std::memcpy(B.h_jobs.p, B.jobs.data(), B.n_jobs * sizeof(DJob));
  CK(cudaMemcpyAsync(B.d_jobs.p, B.h_jobs.p, B.n_jobs * sizeof(DJob), cudaMemcpyHostToDevice, ctx->stream));
  if (!B.job_mats.empty())
    CK(cudaMemcpyAsync(B.d_job_mats.p, B.job_mats.data(), B.job_mats.size() * sizeof(DMat), cudaMemcpyHostToDevice,
                       ctx->stream));
  if (!B.panels.empty())
    CK(cudaMemcpyAsync(B.d_panels.p, B.panels.data(), B.panels.size() * sizeof(DPanel), cudaMemcpyHostToDevice,
                       ctx->stream));
  if (!B.groups.empty())
    CK(cudaMemcpyAsync(B.d_groups.p, B.groups.data(), B.groups.size() * sizeof(DPanelGroup), cudaMemcpyHostToDevice,
                       ctx->stream));
  CK(cudaMemcpyAsync(B.d_rjobs.p, B.rjobs.data(), B.n_jobs * sizeof(DReverbJob), cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return OMG_OK;
}

// The device-side work of one launch (recorded into a graph).
// part 1: clear the scratch and trace; part 2: finalize and reverb.
int32_t record_launch(omg_ctx* ctx, BatchRec& B, cudaStream_t s, int parts = 3) {
  if (parts & 1) {
    CK(cudaMemsetAsync(B.d_hdr.p, 0, sizeof(DLaunch), s));
    CK(cudaMemsetAsync(B.d_acc.p, 0, B.n_acc * sizeof(float), s));
    CK(cudaMemsetAsync(B.d_seg.p, 0, B.n_jobs * sizeof(uint32_t), s));
    CK(cudaMemsetAsync(B.d_ep_ctl.p, 0, (kMaxEpochs + 1) * sizeof(EpochCtl), s));
    // cooperative walks need the near-tie rule and a 4-wide tree in every scene
    LaunchShape eff = B.shape;
    eff.loop_guard = ctx->prm.loop_guard;
    if (eff.mode == 2 && !B.coop_ok) eff.mode = 0;
    if (eff.tail_mode == 2 && !B.coop_ok) eff.tail_mode = 0;
    CK(launch_wavefront(B.d_jobs.p, B.n_jobs, B.total_rays, B.max_nb, ctx->d_scenes.p, B.d_job_mats.p,
                        B.d_panels.p, B.d_groups.p, B.d_acc.p, B.d_hdr.p, B.d_seg.p, B.wf, B.d_ep_q.p,
                        B.d_ep_ctl.p, eff, ctx->n_sms, ctx->prm.tie_mode != 0, s,
                        ctx->prm.tri_test == OMG_TRI_WATERTIGHT));
  }
  if (parts & 2) {
    CK(launch_finalize(B.d_jobs.p, B.n_jobs, B.d_acc.p, B.d_out.p, B.n_out, s));
    CK(launch_reverb(B.d_rjobs.p, B.n_jobs, B.max_bins, B.d_out.p, B.d_reverb.p, B.d_seg.p, s));
  }
  return OMG_OK;
}

int32_t record_readback(omg_ctx* ctx, BatchRec& B, cudaStream_t s) {
  CK(cudaMemcpyAsync(B.h_out.p, B.d_out.p, B.n_out * sizeof(float), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(B.h_reverb.p, B.d_reverb.p, B.n_jobs * sizeof(omg_reverb), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(B.h_hdr.p, B.d_hdr.p, sizeof(DLaunch), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(B.h_seg.p, B.d_seg.p, B.n_jobs * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  return OMG_OK;
}

// Record the batch's work into one executable graph on capture stream cs.
int32_t capture_graph(omg_ctx* ctx, BatchRec& B, cudaStream_t cs, bool io, int parts, cudaGraphExec_t* out) {
  cudaGraph_t g;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return fail(ctx, e, "cudaStreamBeginCapture");
  int32_t rc = OMG_OK;
  if (io) {
    e = cudaMemcpyAsync(B.d_jobs.p, B.h_jobs.p, B.n_jobs * sizeof(DJob), cudaMemcpyHostToDevice, cs);
    if (e != cudaSuccess) rc = fail(ctx, e, "cudaMemcpyAsync jobs");
  }
  if (rc == OMG_OK) rc = record_launch(ctx, B, cs, parts);
  if (rc == OMG_OK && io) rc = record_readback(ctx, B, cs);
  e = cudaStreamEndCapture(cs, &g);
  if (rc != OMG_OK) return rc;
  if (e != cudaSuccess) return fail(ctx, e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(ctx, e, "cudaGraphInstantiate");
  return OMG_OK;
}

int32_t build_graphs(omg_ctx* ctx, BatchRec& B) {
  for (cudaGraphExec_t* g : {&B.graph, &B.graph_io, &B.graph_a, &B.graph_b}) {
    if (*g) cudaGraphExecDestroy(*g);
    *g = nullptr;
  }
  cudaStream_t cs;
  CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  int32_t rc = capture_graph(ctx, B, cs, false, 3, &B.graph);
  if (rc == OMG_OK) rc = capture_graph(ctx, B, cs, true, 3, &B.graph_io);
  if (rc == OMG_OK) rc = capture_graph(ctx, B, cs, false, 1, &B.graph_a);
  if (rc == OMG_OK) rc = capture_graph(ctx, B, cs, false, 2, &B.graph_b);
  cudaStreamDestroy(cs);
  return rc;
}

int32_t prepare_batch(omg_ctx* ctx, BatchRec& B, const omg_job* jobs, uint32_t n_jobs, const omg_panel* panels,
                      uint32_t n_panels) {
  B.shape = ctx->shape;
  int32_t rc = fill_batch(ctx, B, jobs, n_jobs, panels, n_panels);
  if (rc) return rc;
  if ((rc = alloc_batch(ctx, B))) return rc;
  if ((rc = upload_batch(ctx, B))) return rc;
  if ((rc = build_graphs(ctx, B))) return rc;
  B.signature = batch_signature(jobs, n_jobs, n_panels, ctx->prm);
  return OMG_OK;
}

int32_t check_kernel_flags(omg_ctx* ctx, const BatchRec& B) {
  ctx->last_flags = B.h_hdr.p->error;
  if (B.h_hdr.p->error) {
    ctx->last_error = "trace kernel: traversal stack, walk budget or loop guard exceeded (flags " +
                      std::to_string(B.h_hdr.p->error) + ")";
    return OMG_E_OVERFLOW;
  }
  return OMG_OK;
}

// The jobs' echograms from the pinned staging arrays into the caller's
// buffers. Large results are copied by a few threads, job by job (one thread
// copies at about 17 GB/s into freshly mapped pages).
void copy_results(const BatchRec& B, float* bins, float* dirs, omg_reverb* reverb) {
  std::vector<uint64_t> bo(B.n_jobs), dof(B.n_jobs);
  uint64_t b = 0, d = 0;
  for (uint32_t i = 0; i < B.n_jobs; i++) {
    bo[i] = b;
    dof[i] = d;
    b += (uint64_t)B.jobs[i].n_bins * B.jobs[i].nb;
    d += (uint64_t)B.jobs[i].n_bins * 3;
  }
  const int threads = (b + d) * sizeof(float) >= (1u << 20) ? 4 : 1;
#pragma omp parallel for num_threads(threads) schedule(static)
  for (int64_t i = 0; i < (int64_t)B.n_jobs; i++) {
    const DJob& j = B.jobs[i];
    const uint64_t nbb = (uint64_t)j.n_bins * j.nb, nd = (uint64_t)j.n_bins * 3;
    if (bins) std::memcpy(bins + bo[i], B.h_out.p + j.out_off, nbb * sizeof(float));
    if (dirs) std::memcpy(dirs + dof[i], B.h_out.p + j.out_off + nbb, nd * sizeof(float));
  }
  if (reverb) {
    std::memcpy(reverb, B.h_reverb.p, B.n_jobs * sizeof(omg_reverb));
    for (uint32_t i = 0; i < B.n_jobs; i++) reverb[i].segments = B.h_seg.p[i];
  }
}

// One synchronous pass through the io graph: H2D jobs, launch, D2H, bounded wait.
int32_t run_io(omg_ctx* ctx, BatchRec& B, float* bins, float* dirs, omg_reverb* reverb) {
  std::memcpy(B.h_jobs.p, B.jobs.data(), B.n_jobs * sizeof(DJob));
  ctx->last_h2d += B.n_jobs * sizeof(DJob);
  ctx->last_d2h = B.n_out * sizeof(float) + B.n_jobs * (sizeof(omg_reverb) + sizeof(uint32_t)) + sizeof(DLaunch);
  CK(cudaGraphLaunch(B.graph_io, ctx->stream));
  CK(cudaEventRecord(B.done, ctx->stream));
  int32_t rc = wait_event(ctx, B.done, timeout_of(ctx));
  if (rc) return rc;
  if ((rc = check_kernel_flags(ctx, B))) return rc;
  copy_results(B, bins, dirs, reverb);
  return OMG_OK;
}

// New per-job values into a batch whose job layout is unchanged: the job
// array is refilled (it travels with each launch), materials and panels are
// re-uploaded only when they differ, graphs are rebuilt on a shape change.
int32_t refill_batch(omg_ctx* ctx, BatchRec& B, const omg_job* jobs, uint32_t n_jobs, const omg_panel* panels,
                     uint32_t n_panels) {
  std::vector<DMat> old_mats = B.job_mats;
  std::vector<DPanel> old_panels = B.panels;
  int32_t rc = fill_batch(ctx, B, jobs, n_jobs, panels, n_panels);
  if (rc) return rc;
  // materials and panels change rarely: re-upload only when they differ
  bool mats_same = old_mats.size() == B.job_mats.size() &&
                   std::memcmp(old_mats.data(), B.job_mats.data(), old_mats.size() * sizeof(DMat)) == 0;
  bool pan_same = old_panels.size() == B.panels.size() &&
                  std::memcmp(old_panels.data(), B.panels.data(), old_panels.size() * sizeof(DPanel)) == 0;
  if (!mats_same && !B.job_mats.empty()) ctx->last_h2d += B.job_mats.size() * sizeof(DMat);
  if (!pan_same && !B.panels.empty()) ctx->last_h2d += B.panels.size() * sizeof(DPanel);
  if (!mats_same && !B.job_mats.empty())
    CK(cudaMemcpyAsync(B.d_job_mats.p, B.job_mats.data(), B.job_mats.size() * sizeof(DMat),
                       cudaMemcpyHostToDevice, ctx->stream));
  if (!pan_same && !B.panels.empty()) {
    CK(cudaMemcpyAsync(B.d_panels.p, B.panels.data(), B.panels.size() * sizeof(DPanel), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaMemcpyAsync(B.d_groups.p, B.groups.data(), B.groups.size() * sizeof(DPanelGroup),
                       cudaMemcpyHostToDevice, ctx->stream));
  }
  // the context's launch shape changed since the graphs were recorded
  if (std::memcmp(&B.shape, &ctx->shape, sizeof(LaunchShape)) != 0) {
    B.shape = ctx->shape;
    if ((rc = build_graphs(ctx, B))) return rc;
  }
  return OMG_OK;
}

// Synchronous one-shot through the context's cached batch (rebuilt only when
// the job layout changes; per-call values travel in the job array).
int32_t one_shot(omg_ctx* ctx, const omg_job* jobs, uint32_t n_jobs, const omg_panel* panels, uint32_t n_panels,
                 float* bins, float* dirs, omg_reverb* reverb) {
  ctx->last_h2d = 0;
  uint64_t sig = batch_signature(jobs, n_jobs, n_panels, ctx->prm);
  if (!ctx->cached || ctx->cached->signature != sig) {
    ctx->cached.reset(new BatchRec());
    int32_t rc = prepare_batch(ctx, *ctx->cached, jobs, n_jobs, panels, n_panels);
    if (rc) {
      ctx->cached.reset();
      return rc;
    }
  } else {
    int32_t rc = refill_batch(ctx, *ctx->cached, jobs, n_jobs, panels, n_panels);
    if (rc) return rc;
  }
  return run_io(ctx, *ctx->cached, bins, dirs, reverb);
}

void job_from_world(omg_job& j, uint32_t scene_id, const omg_world_job& w, uint32_t n_panels) {
  std::memset(&j, 0, sizeof(j));
  j.geom = OMG_GEOM_MESH;
  j.scene_id = scene_id;
  for (int k = 0; k < 3; k++) {
    j.src[k] = w.src[k];
    j.lis[k] = w.lis[k];
  }
  j.n_rays = w.n_rays;
  for (int b = 0; b < OMG_MAX_BANDS; b++) j.energy[b] = w.energy[b];
  j.seed = w.seed;
  j.n_panels = n_panels;
}

}  // namespace

namespace omg {

int32_t batch_prepare(omg_ctx* ctx, BatchRec& B, const omg_job* jobs, uint32_t n_jobs, const omg_panel* panels,
                      uint32_t n_panels) {
  return prepare_batch(ctx, B, jobs, n_jobs, panels, n_panels);
}
int32_t batch_refill(omg_ctx* ctx, BatchRec& B, const omg_job* jobs, uint32_t n_jobs, const omg_panel* panels,
                     uint32_t n_panels) {
  return refill_batch(ctx, B, jobs, n_jobs, panels, n_panels);
}
uint64_t batch_layout(const omg_job* jobs, uint32_t n_jobs, uint32_t n_panels, const omg_params& P) {
  return batch_signature(jobs, n_jobs, n_panels, P);
}
int32_t batch_flags(omg_ctx* ctx, const BatchRec& B) { return check_kernel_flags(ctx, B); }

}  // namespace omg

// ====================================================================== C ABI
extern "C" {

void omg_params_default(omg_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->n_bands = 3;
  p->n_bins = 300;
  p->bin_dt = 0.010f;
  p->max_time = 3.0f;
  p->max_bounces = 64;
  p->energy_floor = 1e-7f;
  p->receiver_radius = 0.5f;
  p->wall_eps = 1e-3f;
  p->speed_of_sound = 343.0f;
  p->dir_band = 1;
  p->device = 0;
  p->timeout_ms = 10000;
  p->tie_mode = 0;
}

int32_t omg_abi_version(void) { return OMG_ABI_VERSION; }

const char* omg_status_string(int32_t s) {
  switch (s) {
    case OMG_OK: return "ok";
    case OMG_PENDING: return "pending";
    case OMG_E_INVALID: return "invalid argument";
    case OMG_E_OOM: return "out of memory";
    case OMG_E_DEVICE: return "device error";
    case OMG_E_TIMEOUT: return "timeout";
    case OMG_E_OVERFLOW: return "traversal overflow";
    case OMG_E_NOT_FOUND: return "not found";
    case OMG_E_NO_DEVICE: return "no device";
    default: return "unknown status";
  }
}

const char* omg_last_error(const omg_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

uint32_t omg_last_flags(const omg_ctx* ctx) { return ctx ? ctx->last_flags : 0u; }

int32_t omg_set_limits(omg_ctx* ctx, uint32_t walk_budget, uint32_t loop_guard) {
  if (!ctx) return OMG_E_INVALID;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, cudaGetLastError(), "cudaSetDevice");
  // nothing of this context may be in flight while its tables and graphs change
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->prm.walk_budget = walk_budget;
  ctx->prm.loop_guard = loop_guard;
  int32_t rc = sync_scene_table(ctx);   // the walk budgets live in the scene records
  if (rc) return rc;
  // the loop guard is a kernel argument recorded in each batch's graphs
  ctx->cached.reset();
  for (auto& kv : ctx->batches)
    if ((rc = build_graphs(ctx, *kv.second))) return rc;
  return OMG_OK;
}

omg_ctx* omg_create(const omg_params* p) {
  omg_params prm;
  if (p) prm = *p;
  else omg_params_default(&prm);
  if (prm.n_bands == 0 || prm.n_bands > OMG_MAX_BANDS || prm.n_bins == 0 || prm.n_bins > kMaxBins ||
      !(prm.bin_dt > 0.0f) ||
      prm.dir_band >= prm.n_bands || !(prm.speed_of_sound > 0.0f) ||
      (prm.tri_test != OMG_TRI_REFERENCE && prm.tri_test != OMG_TRI_WATERTIGHT) ||
      (prm.tri_test == OMG_TRI_WATERTIGHT && prm.tie_mode != 1))
    return nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= prm.device || prm.device < 0) {
    cudaGetLastError();
    return nullptr;
  }
  if (cudaSetDevice(prm.device) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  omg_ctx* ctx = new omg_ctx();
  ctx->prm = prm;
  ctx->device = prm.device;
  cudaDeviceGetAttribute(&ctx->n_sms, cudaDevAttrMultiProcessorCount, prm.device);
  if (cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return nullptr;
  }
  ctx->stream = ctx->own;
  if (sync_scene_table(ctx) != OMG_OK) {
    cudaStreamDestroy(ctx->own);
    delete ctx;
    return nullptr;
  }
  return ctx;
}

void omg_destroy(omg_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ctx->tickets.clear();
  ctx->batches.clear();
  ctx->cached.reset();
  ctx->probes.clear();
  ctx->scenes.clear();
  if (ctx->own) cudaStreamDestroy(ctx->own);
  delete ctx;
}

int32_t omg_set_stream(omg_ctx* ctx, void* s) {
  if (!ctx) return OMG_E_INVALID;
  ctx->stream = s ? (cudaStream_t)s : ctx->own;
  return OMG_OK;
}


// ------------------------------------------------------------------ batches
int32_t omg_batch_create(omg_ctx* ctx, const omg_job* jobs, uint32_t n_jobs, const omg_panel* panels,
                         uint32_t n_panels, uint32_t* batch_id) {
  if (!ctx || !jobs || !n_jobs || !batch_id || (n_panels && !panels)) return OMG_E_INVALID;
  std::unique_ptr<BatchRec> B(new BatchRec());
  int32_t rc = prepare_batch(ctx, *B, jobs, n_jobs, panels, n_panels);
  if (rc) return rc;
  *batch_id = ctx->next_batch++;
  ctx->batches[*batch_id] = std::move(B);
  return OMG_OK;
}

int32_t omg_batch_launch(omg_ctx* ctx, uint32_t id) { return omg_batch_launch_part(ctx, id, 0); }

int32_t omg_batch_launch_part(omg_ctx* ctx, uint32_t id, uint32_t part) {
  if (!ctx || part > 2) return OMG_E_INVALID;
  auto it = ctx->batches.find(id);
  if (it == ctx->batches.end()) return OMG_E_NOT_FOUND;
  BatchRec& B = *it->second;
  CK(cudaGraphLaunch(part == 0 ? B.graph : (part == 1 ? B.graph_a : B.graph_b), ctx->stream));
  return OMG_OK;
}

int32_t omg_io_bytes(omg_ctx* ctx, uint64_t* h2d, uint64_t* d2h) {
  if (!ctx) return OMG_E_INVALID;
  if (h2d) *h2d = ctx->last_h2d;
  if (d2h) *d2h = ctx->last_d2h;
  return OMG_OK;
}

int32_t omg_batch_read(omg_ctx* ctx, uint32_t id, float* bins, float* dirs, omg_reverb* reverb) {
  if (!ctx) return OMG_E_INVALID;
  auto it = ctx->batches.find(id);
  if (it == ctx->batches.end()) return OMG_E_NOT_FOUND;
  BatchRec& B = *it->second;
  int32_t rc = record_readback(ctx, B, ctx->stream);
  if (rc) return rc;
  CK(cudaEventRecord(B.done, ctx->stream));
  if ((rc = wait_event(ctx, B.done, timeout_of(ctx)))) return rc;
  if ((rc = check_kernel_flags(ctx, B))) return rc;
  copy_results(B, bins, dirs, reverb);
  return OMG_OK;
}

int32_t omg_batch_sizes(omg_ctx* ctx, uint32_t id, uint64_t* nb, uint64_t* nd) {
  if (!ctx) return OMG_E_INVALID;
  auto it = ctx->batches.find(id);
  if (it == ctx->batches.end()) return OMG_E_NOT_FOUND;
  if (nb) *nb = it->second->n_bin_floats;
  if (nd) *nd = it->second->n_dir_floats;
  return OMG_OK;
}

int32_t omg_batch_segments(omg_ctx* ctx, uint32_t id, uint64_t* segments) {
  if (!ctx || !segments) return OMG_E_INVALID;
  auto it = ctx->batches.find(id);
  if (it == ctx->batches.end()) return OMG_E_NOT_FOUND;
  BatchRec& B = *it->second;
  CK(cudaMemcpyAsync(B.h_seg.p, B.d_seg.p, B.n_jobs * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaEventRecord(B.done, ctx->stream));
  int32_t rc = wait_event(ctx, B.done, timeout_of(ctx));
  if (rc) return rc;
  uint64_t s = 0;
  for (uint32_t i = 0; i < B.n_jobs; i++) s += B.h_seg.p[i];
  *segments = s;
  return OMG_OK;
}

int32_t omg_batch_destroy(omg_ctx* ctx, uint32_t id) {
  if (!ctx) return OMG_E_INVALID;
  auto it = ctx->batches.find(id);
  if (it == ctx->batches.end()) return OMG_E_NOT_FOUND;
  cudaStreamSynchronize(ctx->stream);
  ctx->batches.erase(it);
  return OMG_OK;
}

int32_t omg_batch_kernel_count(omg_ctx* ctx, uint32_t id, uint32_t* n) {
  if (!ctx || !n) return OMG_E_INVALID;
  auto it = ctx->batches.find(id);
  if (it == ctx->batches.end()) return OMG_E_NOT_FOUND;
  // finalize, reverb; the persistent kernel once per epoch; wavefront: init,
  // 2 per round, hand-over
  const LaunchShape& sh = it->second->shape;
  const uint32_t epochs = sh.epochs == 0 ? 1u : std::min<uint32_t>(sh.epochs, kMaxEpochs);
  *n = 2 + epochs + (sh.wf_iters ? 2 + 2 * sh.wf_iters : 0);
  return OMG_OK;
}

// ------------------------------------------------------------------ tracing
int32_t omg_trace_box(omg_ctx* ctx, const omg_box_job* job, float* bins, float* dirs, omg_reverb* reverb) {
  if (!ctx || !job) return OMG_E_INVALID;
  omg_job j;
  std::memset(&j, 0, sizeof(j));
  j.geom = OMG_GEOM_BOX;
  for (int k = 0; k < 3; k++) {
    j.box_size[k] = job->size[k];
    j.src[k] = job->src[k];
    j.lis[k] = job->lis[k];
  }
  for (int w = 0; w < 6; w++) j.box_walls[w] = job->walls[w];
  j.n_rays = job->n_rays;
  for (int b = 0; b < OMG_MAX_BANDS; b++) j.energy[b] = job->energy[b];
  j.seed = job->seed;
  return one_shot(ctx, &j, 1, nullptr, 0, bins, dirs, reverb);
}

int32_t omg_trace_world(omg_ctx* ctx, uint32_t scene_id, const omg_world_job* job, const omg_panel* panels,
                        uint32_t n_panels, float* bins, float* dirs, omg_reverb* reverb) {
  if (!ctx || !job || (n_panels && !panels)) return OMG_E_INVALID;
  omg_job j;
  job_from_world(j, scene_id, *job, n_panels);
  return one_shot(ctx, &j, 1, panels, n_panels, bins, dirs, reverb);
}

int32_t omg_trace_batch(omg_ctx* ctx, const omg_job* jobs, uint32_t n_jobs, const omg_panel* panels,
                        uint32_t n_panels, float* bins, float* dirs, omg_reverb* reverb) {
  if (!ctx || !jobs || !n_jobs || (n_panels && !panels)) return OMG_E_INVALID;
  return one_shot(ctx, jobs, n_jobs, panels, n_panels, bins, dirs, reverb);
}

// ------------------------------------------------------------ async tickets
int32_t omg_submit_world(omg_ctx* ctx, uint32_t scene_id, const omg_world_job* job, const omg_panel* panels,
                         uint32_t n_panels, uint32_t* ticket) {
  if (!ctx || !job || !ticket || (n_panels && !panels)) return OMG_E_INVALID;
  omg_job j;
  job_from_world(j, scene_id, *job, n_panels);
  Ticket t;
  t.batch.reset(new BatchRec());
  int32_t rc = prepare_batch(ctx, *t.batch, &j, 1, panels, n_panels);
  if (rc) return rc;
  BatchRec& B = *t.batch;
  std::memcpy(B.h_jobs.p, B.jobs.data(), sizeof(DJob));
  CK(cudaGraphLaunch(B.graph_io, ctx->stream));
  CK(cudaEventRecord(B.done, ctx->stream));
  *ticket = ctx->next_ticket++;
  ctx->tickets[*ticket] = std::move(t);
  return OMG_OK;
}

int32_t omg_poll(omg_ctx* ctx, uint32_t ticket, float* bins, float* dirs, omg_reverb* reverb) {
  if (!ctx) return OMG_E_INVALID;
  auto it = ctx->tickets.find(ticket);
  if (it == ctx->tickets.end()) return OMG_E_NOT_FOUND;
  BatchRec& B = *it->second.batch;
  cudaError_t q = cudaEventQuery(B.done);
  if (q == cudaErrorNotReady) return OMG_PENDING;
  if (q != cudaSuccess) return fail(ctx, q, "cudaEventQuery");
  int32_t rc = check_kernel_flags(ctx, B);
  if (rc == OMG_OK) copy_results(B, bins, dirs, reverb);
  ctx->tickets.erase(it);
  return rc;
}

// ---------------------------------------------------------------- autotuner
namespace {

// Mean time of the clear + trace part with the batch's current shape: the part
// is recorded into a graph (as launches run it), launched once to warm up,
// then `reps` times between two events on the context stream.
int32_t time_trace(omg_ctx* ctx, BatchRec& B, uint32_t reps, cudaStream_t cs, cudaEvent_t e0, cudaEvent_t e1,
                   float* ms) {
  cudaGraphExec_t g = nullptr;
  int32_t rc = capture_graph(ctx, B, cs, false, 1, &g);
  if (rc) return rc;
  cudaError_t e = cudaGraphLaunch(g, ctx->stream);
  if (e == cudaSuccess) e = cudaEventRecord(e0, ctx->stream);
  for (uint32_t r = 0; r < reps && e == cudaSuccess; r++) e = cudaGraphLaunch(g, ctx->stream);
  if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
  if (e != cudaSuccess) rc = fail(ctx, e, "autotune launch");
  if (rc == OMG_OK) rc = wait_event(ctx, e1, timeout_of(ctx) * (reps + 1));
  if (rc == OMG_OK) {
    cudaEventElapsedTime(ms, e0, e1);
    *ms /= (float)reps;
  }
  cudaGraphExecDestroy(g);
  return rc;
}

void shape_to_result(const LaunchShape& sh, float ms, omg_tune_result* r) {
  r->block_threads = sh.block_threads;
  r->blocks_per_sm = sh.blocks_per_sm;
  r->refill_min = sh.refill_min;
  r->walk_steps = sh.walk_steps;
  r->wf_rounds = sh.wf_iters;
  r->wf_tail = sh.wf_tail;
  r->epochs = sh.epochs;
  r->park_pct = sh.park_pct;
  r->shade_min = sh.shade_min;
  r->mode = sh.mode;
  r->tail_mode = sh.tail_mode;
  r->wide = sh.wide;
  r->wl_shade_min = sh.wl_shade_min;
  r->ms = ms;
}

}  // namespace

// Four stages: the persistent kernel's shape alone (one launch), then epoch
// counts and park thresholds with that shape, then the wavefront kernels'
// shading group (when the best shape runs one), then wavefront round counts
// and hand-over thresholds in front of the best of those.
int32_t omg_batch_autotune(omg_ctx* ctx, uint32_t id, uint32_t reps, omg_tune_result* best) {
  if (!ctx || !best) return OMG_E_INVALID;
  auto it = ctx->batches.find(id);
  if (it == ctx->batches.end()) return OMG_E_NOT_FOUND;
  BatchRec& B = *it->second;
  if (reps == 0) reps = 3;
  const uint32_t threads[] = {128, 256};
  const uint32_t per_sm[] = {2, 4, 8};
  const uint32_t refill[] = {1, 8};
  const uint32_t walks[] = {0, 8, 32};
  const uint32_t shade_mins[] = {1, 16, 32};
  const uint32_t wl_walks[] = {0, 4, 8, 16, 32};
  const uint32_t rounds[] = {16, 32, 48, 64, 96, 128, 192};
  const uint32_t tails[] = {0, 2048, 8192, 32768};
  const uint32_t epoch_counts[] = {2, 3, 4, 8};
  const uint32_t park_pcts[] = {5, 10, 20, 40};
  const uint32_t tail_modes[] = {0, 2};
  const uint32_t wl_shades[] = {1, 4, 8, 16};
  cudaEvent_t e0, e1;
  cudaStream_t cs;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  const LaunchShape keep = B.shape;
  float best_ms = 1e30f;
  LaunchShape best_shape = keep;
  int32_t rc = OMG_OK;
  auto try_shape = [&](const LaunchShape& sh) -> int32_t {
    B.shape = sh;
    float ms = 0.0f;
    int32_t r = time_trace(ctx, B, reps, cs, e0, e1, &ms);
    if (r == OMG_OK && ms < best_ms) {
      best_ms = ms;
      best_shape = sh;
    }
    return r;
  };
  for (uint32_t th : threads)
    for (uint32_t ps : per_sm) {
      for (uint32_t rf : refill)
        for (uint32_t wk : walks)
          for (uint32_t sm : shade_mins) {
            if (rc || th * ps > 2048) continue;
            LaunchShape sh;
            sh.block_threads = th;
            sh.blocks_per_sm = ps;
            sh.refill_min = rf;
            sh.walk_steps = wk;
            sh.shade_min = sm;
            rc = try_shape(sh);
          }
      for (uint32_t wk : wl_walks) {
        if (rc || th * ps > 2048) continue;
        LaunchShape sh;
        sh.mode = 1;
        sh.block_threads = th;
        sh.blocks_per_sm = ps;
        sh.walk_steps = wk;
        rc = try_shape(sh);
        if (rc || !B.coop_ok || th != 256) continue;
        sh.mode = 2;
        rc = try_shape(sh);
      }
    }
  // the same persistent kernel walking the 4-wide tree (near-tie rule, every
  // scene host-built): fewer dependent steps per walk, which pays where the
  // walks wait on memory (trees beyond L2)
  if (B.coop_ok && best_shape.mode != 2) {
    const LaunchShape base = best_shape;
    for (uint32_t wk : walks) {
      if (rc) continue;
      LaunchShape sh = base;
      sh.wide = 1;
      sh.walk_steps = wk;
      rc = try_shape(sh);
    }
  }
  const LaunchShape persistent = best_shape;
  for (uint32_t tm : tail_modes)
    for (uint32_t ne : epoch_counts)
      for (uint32_t pp : park_pcts) {
        if (rc || (tm == 2 && !B.coop_ok)) continue;
        LaunchShape sh = persistent;
        sh.epochs = ne;
        sh.park_pct = pp;
        sh.tail_mode = tm;
        rc = try_shape(sh);
      }
  // the shading group of the wavefront kernels (modes 1 and 2), where the
  // best shape so far runs one of them
  const LaunchShape grouped = best_shape;
  if (grouped.mode != 0 || (grouped.epochs > 1 && grouped.tail_mode != 0))
    for (uint32_t ws : wl_shades) {
      if (rc) continue;
      LaunchShape sh = grouped;
      sh.wl_shade_min = ws;
      rc = try_shape(sh);
    }
  const LaunchShape chained = best_shape;
  for (uint32_t nr : rounds)
    for (uint32_t tl : tails) {
      if (rc) continue;
      LaunchShape sh = chained;
      sh.wf_iters = nr;
      sh.wf_tail = tl;
      rc = try_shape(sh);
    }
  cudaStreamDestroy(cs);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  B.shape = rc == OMG_OK ? best_shape : keep;
  if (rc) return rc;
  if ((rc = build_graphs(ctx, B))) return rc;
  ctx->shape = best_shape;
  shape_to_result(best_shape, best_ms, best);
  return OMG_OK;
}

// Set the launch shape of a batch (and the default of later batches) by hand.
int32_t omg_batch_set_shape(omg_ctx* ctx, uint32_t id, const omg_tune_result* shape) {
  if (!ctx || !shape) return OMG_E_INVALID;
  auto it = ctx->batches.find(id);
  if (it == ctx->batches.end()) return OMG_E_NOT_FOUND;
  if (shape->block_threads == 0 || shape->block_threads % 32 != 0 || shape->block_threads > 256 ||
      shape->blocks_per_sm == 0 || shape->block_threads * shape->blocks_per_sm > 2048 || shape->refill_min == 0 ||
      shape->refill_min > 32 || shape->wf_rounds > 4096 || shape->epochs > kMaxEpochs || shape->park_pct > 100 ||
      shape->shade_min > 32 || shape->mode > 2 || shape->tail_mode > 2 || shape->wl_shade_min > 32)
    return OMG_E_INVALID;
  BatchRec& B = *it->second;
  LaunchShape sh;
  sh.block_threads = shape->block_threads;
  sh.blocks_per_sm = shape->blocks_per_sm;
  sh.refill_min = shape->refill_min;
  sh.walk_steps = shape->walk_steps;
  sh.wf_iters = shape->wf_rounds;
  sh.wf_tail = shape->wf_tail;
  sh.epochs = shape->epochs;
  sh.park_pct = shape->park_pct;
  sh.shade_min = shape->shade_min == 0 ? 1u : shape->shade_min;
  sh.mode = shape->mode;
  sh.tail_mode = shape->tail_mode;
  sh.wide = shape->wide ? 1u : 0u;
  sh.wl_shade_min = shape->wl_shade_min == 0 ? 32u : shape->wl_shade_min;
  B.shape = sh;
  int32_t rc = build_graphs(ctx, B);
  if (rc) return rc;
  ctx->shape = sh;
  return OMG_OK;
}

int32_t omg_batch_get_shape(omg_ctx* ctx, uint32_t id, omg_tune_result* shape) {
  if (!ctx || !shape) return OMG_E_INVALID;
  auto it = ctx->batches.find(id);
  if (it == ctx->batches.end()) return OMG_E_NOT_FOUND;
  shape_to_result(it->second->shape, 0.0f, shape);
  return OMG_OK;
}

}  // extern "C"
