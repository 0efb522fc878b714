// Wavefront rounds of the path tracer.
//
// A batch holds a few hundred thousand rays of 50 segments on average and up
// to max_bounces. In the persistent kernel each lane owns a ray until it
// ends; once the ray queue is drained, warps run with a handful of live lanes
// for most of the launch. The wavefront form keeps the live rays packed
// instead: each round is
//   extend : closest hit of every live ray (mesh_closest only, few registers)
//   shade  : receiver test, advance, absorb / transmit / scatter
//            (shade_segment, the same code the persistent kernel runs) and a
//            warp-aggregated append of the survivors to the other queue
// over a queue of live ray ids, with the bounce-loop state of each ray
// (position, direction, distance, band energies, stream state, bounce count)
// kept in per-ray records in HBM between the kernels. Rounds are recorded
// once into the batch's CUDA graph; once at most `wf_tail` rays are alive (or
// after `wf_iters` rounds) the remaining rounds return at once and the
// persistent kernel (trace.cu) finishes the tail from the saved state.
//
// Every ray follows exactly the operations of the reference's bounce loop
// (tracer.rs:103-200) in the same order whichever kernel runs a segment, so
// the result is the same as the persistent kernel's alone: only the order of
// the histogram atomics differs, as it does between any two launches.
#include "shade_common.cuh"

namespace omg {

namespace {

constexpr unsigned FULL = 0xffffffffu;

template <int NB>
__device__ __forceinline__ void wf_store_e(const WfState& st, uint32_t r, const float (&e)[NB]) {
  float v[8];
#pragma unroll
  for (int b = 0; b < 8; b++) v[b] = b < NB ? e[b] : 0.0f;
  st.e[r] = make_float4(v[0], v[1], v[2], v[3]);
  if (NB > 4) st.e[st.cap + r] = make_float4(v[4], v[5], v[6], v[7]);
}

// Start every ray (tracer.rs:96-102): stream, direction, source, energies.
template <int NB>
__global__ void wf_init_kernel(const DJob* __restrict__ jobs, uint32_t n_jobs, uint32_t total_rays, WfState st) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r == 0) {
    WfCtl* c = st.ctl;
    c->count[0] = total_rays;
    c->count[1] = 0;
    c->tail = 0;
    c->tail_q = 0;
    c->tail_n = 0;
  }
  if (r >= total_rays) return;
  const uint32_t ji = find_job(jobs, n_jobs, r);
  const DJob& J = jobs[ji];
  Pcg rng;
  rng.init(J.seed, r - J.ray_base);
  float dx, dy, dz;
  unit_sphere(rng, dx, dy, dz);
  st.pos[r] = make_float4(J.src[0], J.src[1], J.src[2], 0.0f);
  st.dir[r] = make_float4(dx, dy, dz, __uint_as_float(rng.s));
  float e[NB];
#pragma unroll
  for (int b = 0; b < NB; b++) e[b] = J.e0[b];
  wf_store_e<NB>(st, r, e);
  st.bounce[r] = 0;
  st.queue[r] = r;
}

// Closest mesh hit of every ray in queue `cur`. The first round that finds at
// most `tail_min` live rays hands them to the persistent kernel; every later
// round then returns at once.
template <bool TIE>
__global__ void __launch_bounds__(256) wf_extend_kernel(const DJob* __restrict__ jobs, uint32_t n_jobs,
                                                        const DScene* __restrict__ scenes, WfState st, uint32_t cur,
                                                        uint32_t tail_min, uint32_t* err) {
  WfCtl* ctl = st.ctl;
  if (ctl->tail) return;
  const uint32_t n = ctl->count[cur];
  if (n <= tail_min) {
    // every block of this launch takes the same branch: n is read-only here
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      ctl->tail_q = cur;
      ctl->tail_n = n;
      ctl->tail = 1;
    }
    return;
  }
  // the queue this round's shading appends to
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->count[cur ^ 1u] = 0;
  const uint32_t* __restrict__ q = st.queue + (size_t)cur * st.cap;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const uint32_t r = q[k];
    const DJob& J = jobs[find_job(jobs, n_jobs, r)];
    if (J.geom != OMG_GEOM_MESH) continue;   // shoeboxes are hit analytically in shade
    const DScene S = scenes[J.scene];
    const float4 P = st.pos[r], D = st.dir[r];
    float t = FLT_MAX;
    int prim = -1;
    const bool have = (TIE && S.nodes4) ? mesh_closest4(S, P.x, P.y, P.z, D.x, D.y, D.z, t, prim, err)
                                        : mesh_closest<TIE>(S, P.x, P.y, P.z, D.x, D.y, D.z, t, prim, err);
    st.hit[r] = make_float2(t, __int_as_float(have ? prim : -1));
  }
}

// One segment of every ray in queue `cur` (tracer.rs:103-200); survivors go
// to queue cur ^ 1, finished rays add their segment count to their job.
template <int NB>
__global__ void __launch_bounds__(256) wf_shade_kernel(const DJob* __restrict__ jobs, uint32_t n_jobs,
                                                       const DScene* __restrict__ scenes,
                                                       const DMat* __restrict__ job_mats,
                                                       const DPanel* __restrict__ panels,
                                                       const DPanelGroup* __restrict__ groups,
                                                       float* __restrict__ acc, WfState st, uint32_t cur,
                                                       uint32_t* __restrict__ job_segments) {
  WfCtl* ctl = st.ctl;
  if (ctl->tail) return;
  const uint32_t n = ctl->count[cur];
  const uint32_t* __restrict__ q = st.queue + (size_t)cur * st.cap;
  uint32_t* __restrict__ qn = st.queue + (size_t)(cur ^ 1u) * st.cap;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t stride = gridDim.x * blockDim.x;
  // warp-uniform trip count: the append ballot needs the whole warp
  for (uint32_t k0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); k0 < n; k0 += stride) {
    const uint32_t k = k0 + lane;
    bool alive = false;
    uint32_t r = 0;
    if (k < n) {
      r = q[k];
      const uint32_t ji = find_job(jobs, n_jobs, r);
      const DJob& J = jobs[ji];
      const float4 P = st.pos[r], D = st.dir[r];
      float px = P.x, py = P.y, pz = P.z, dist = P.w;
      float dx = D.x, dy = D.y, dz = D.z;
      Pcg rng;
      rng.s = __float_as_uint(D.w);
      float e[NB];
      {
        const float4 e0 = st.e[r];
        const float4 e1 = NB > 4 ? st.e[st.cap + r] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const float ev[8] = {e0.x, e0.y, e0.z, e0.w, e1.x, e1.y, e1.z, e1.w};
#pragma unroll
        for (int b = 0; b < NB; b++) e[b] = ev[b];
      }
      uint32_t bounce = st.bounce[r];
      Hit h;
      h.t = FLT_MAX;
      h.m = nullptr;
      bool have;
      if (J.geom == OMG_GEOM_BOX) {
        have = box_hit(J, job_mats, px, py, pz, dx, dy, dz, h);
      } else {
        const float2 H = st.hit[r];
        const int prim = __float_as_int(H.y);
        have = prim >= 0;
        if (have) {
          const DScene& S = scenes[J.scene];
          const float4 p0 = __ldg(S.prims + 3 * prim + 0);
          const float4 p1 = __ldg(S.prims + 3 * prim + 1);
          const float4 nn = __ldg(S.normals + __float_as_uint(p1.w));
          float nx = nn.x, ny = nn.y, nz = nn.z;
          if (nx * dx + ny * dy + nz * dz > 0.0f) { nx = nx * -1.0f; ny = ny * -1.0f; nz = nz * -1.0f; }
          h.t = H.x;
          h.nx = nx; h.ny = ny; h.nz = nz;
          h.m = S.mats + __float_as_uint(p0.w);
        }
      }
      if (J.n_groups) have = panels_hit(J, panels, groups, job_mats, px, py, pz, dx, dy, dz, have, h);
      const float t_hit = have ? h.t : FLT_MAX;
      bool done = shade_segment<NB>(J, acc, h, have, t_hit, px, py, pz, dx, dy, dz, dist, e, rng);
      bounce++;
      if (!done && bounce >= J.max_bounces) done = true;
      if (done) {
        atomicAdd(job_segments + ji, bounce);
      } else {
        st.pos[r] = make_float4(px, py, pz, dist);
        st.dir[r] = make_float4(dx, dy, dz, __uint_as_float(rng.s));
        wf_store_e<NB>(st, r, e);
        st.bounce[r] = bounce;
        alive = true;
      }
    }
    const unsigned m = __ballot_sync(FULL, alive);
    if (m) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(&ctl->count[cur ^ 1u], (uint32_t)__popc(m));
      base = __shfl_sync(FULL, base, 0);
      if (alive) qn[base + (uint32_t)__popc(m & ((1u << lane) - 1u))] = r;
    }
  }
}

// After the last recorded round: copy the live rays' ids into the first
// epoch's queue (from the hand-over queue, or the queue the next round would
// have read).
__global__ void wf_handover_kernel(WfState st, uint32_t q_next, uint32_t* __restrict__ ep_q0, EpochCtl* ep0) {
  const WfCtl* ctl = st.ctl;
  const bool tail = ctl->tail != 0u;
  const uint32_t tq = tail ? ctl->tail_q : q_next;
  const uint32_t n = tail ? ctl->tail_n : ctl->count[q_next];
  const uint32_t* __restrict__ q = st.queue + (size_t)tq * st.cap;
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  for (uint32_t i = tid; i < n; i += gridDim.x * blockDim.x) ep_q0[i] = q[i];
  if (tid == 0) ep0->n = n;
}

template <int NB, bool TIE>
cudaError_t launch_rounds(const DJob* jobs, uint32_t n_jobs, uint32_t total_rays, const DScene* scenes,
                          const DMat* job_mats, const DPanel* panels, const DPanelGroup* groups, float* acc,
                          DLaunch* hdr, uint32_t* job_segments, const WfState& st, uint32_t* ep_q, EpochCtl* ep_ctl,
                          const LaunchShape& shape, int n_sms, cudaStream_t s) {
  constexpr uint32_t kThreads = 256;
  const uint32_t need = (total_rays + kThreads - 1) / kThreads;
  wf_init_kernel<NB><<<need, kThreads, 0, s>>>(jobs, n_jobs, total_rays, st);
  // grid-stride rounds: enough blocks for every live ray at full occupancy
  const uint32_t cap_blocks = (uint32_t)n_sms * 8u;
  const uint32_t blocks = need < cap_blocks ? need : cap_blocks;
  for (uint32_t i = 0; i < shape.wf_iters; i++) {
    const uint32_t cur = i & 1u;
    wf_extend_kernel<TIE><<<blocks, kThreads, 0, s>>>(jobs, n_jobs, scenes, st, cur, shape.wf_tail, &hdr->error);
    wf_shade_kernel<NB><<<blocks, kThreads, 0, s>>>(jobs, n_jobs, scenes, job_mats, panels, groups, acc, st, cur,
                                                    job_segments);
  }
  wf_handover_kernel<<<blocks, kThreads, 0, s>>>(st, shape.wf_iters & 1u, ep_q, ep_ctl);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_wavefront(const DJob* jobs, uint32_t n_jobs, uint32_t total_rays, uint32_t max_nb,
                             const DScene* scenes, const DMat* job_mats, const DPanel* panels,
                             const DPanelGroup* groups, float* acc, DLaunch* hdr, uint32_t* job_segments,
                             const WfState& st, uint32_t* ep_q, EpochCtl* ep_ctl, const LaunchShape& shape,
                             int n_sms, bool tie, cudaStream_t s, bool wt) {
  const bool staged = st.ctl && ep_q && ep_ctl && st.cap >= total_rays;
  const bool rounds = staged && shape.wf_iters > 0;
  if (!staged || (!rounds && shape.epochs == 0 && shape.mode == 0))
    return launch_trace(jobs, n_jobs, total_rays, max_nb, scenes, job_mats, panels, groups, acc, hdr, job_segments,
                        shape, n_sms, tie, s, nullptr, wt);
  if (n_jobs == 0 || total_rays == 0) return cudaSuccess;
  if (rounds) {
    cudaError_t e;
    if (max_nb <= 3) {
      e = tie ? launch_rounds<3, true>(jobs, n_jobs, total_rays, scenes, job_mats, panels, groups, acc, hdr,
                                       job_segments, st, ep_q, ep_ctl, shape, n_sms, s)
              : launch_rounds<3, false>(jobs, n_jobs, total_rays, scenes, job_mats, panels, groups, acc, hdr,
                                        job_segments, st, ep_q, ep_ctl, shape, n_sms, s);
    } else {
      e = tie ? launch_rounds<8, true>(jobs, n_jobs, total_rays, scenes, job_mats, panels, groups, acc, hdr,
                                       job_segments, st, ep_q, ep_ctl, shape, n_sms, s)
              : launch_rounds<8, false>(jobs, n_jobs, total_rays, scenes, job_mats, panels, groups, acc, hdr,
                                        job_segments, st, ep_q, ep_ctl, shape, n_sms, s);
    }
    if (e != cudaSuccess) return e;
  }
  // the epoch chain: epoch k reads queue k & 1 and parks into queue (k + 1) & 1
  uint32_t n_ep = shape.epochs == 0 ? 1u : shape.epochs;
  if (n_ep > kMaxEpochs) n_ep = kMaxEpochs;
  for (uint32_t k = 0; k < n_ep; k++) {
    EpochArgs a{};
    a.in_q = (k == 0 && !rounds) ? nullptr : ep_q + (size_t)(k & 1u) * st.cap;
    a.out_q = k + 1 < n_ep ? ep_q + (size_t)((k + 1) & 1u) * st.cap : nullptr;
    a.cur = ep_ctl + k;
    a.next = ep_ctl + k + 1;
    a.park_pct = shape.park_pct;
    a.park_min = shape.park_min;
    a.st = st;
    LaunchShape sk = shape;
    if (k > 0) sk.mode = shape.tail_mode;
    cudaError_t e = launch_trace(jobs, n_jobs, total_rays, max_nb, scenes, job_mats, panels, groups, acc, hdr,
                                 job_segments, sk, n_sms, tie, s, &a, wt);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace omg
