// Stochastic energy path tracer kernels for sm_103a.
//
// One persistent kernel traces every ray of every job of a launch: warps pull
// rays from a global queue and refill idle lanes after each segment, so SIMD
// lanes stay busy while rays end at different bounce counts. Each segment is
// one iteration of the reference's bounce loop (tracer.rs:103-200): closest
// hit, receiver test, then absorb / transmit / scatter.
//
// The same kernel also finishes the rays that the wavefront rounds
// (wavefront.cu) leave alive: it then takes ray ids from the tail queue and
// restores each ray's state instead of starting it.
//
// Arithmetic follows the reference's f32 operation order term by term and
// this file is compiled with -fmad=false, so every f32 result rounds exactly
// as the reference's (and the f32 oracle's) does. The only transcendentals,
// cos/sin of the sphere azimuth, come from the f32 sincos of
// device_common.cuh, which the f32 oracle evaluates identically.
#include "shade_common.cuh"
#include "walk.cuh"

namespace omg {

namespace {

// Up to `steps` node visits / leaf tests; returns true when the walk is done.
template <bool TIE>
__device__ __forceinline__ bool walk_steps(Walk& w, const DScene& S, float ox, float oy, float oz, float dx,
                                           float dy, float dz, int steps, bool wide, uint32_t* err) {
  if (TIE && wide && S.nodes4) return walk4_steps(w, S, ox, oy, oz, dx, dy, dz, steps, err);
  const float4* __restrict__ nodes = S.nodes;
  const float4* __restrict__ prims = S.prims;   // the first-found rule: the reference's test (no watertight context)
  if (!TIE) {
    // the reference's order: each node or leaf as it is reached
    while (steps-- > 0 && w.cur != kDone) {
      if (w.budget-- == 0u) {
        atomicOr(err, 4u);
        w.cur = kDone;
        break;
      }
      if (w.cur >= 0) {
        const float4 n0 = __ldg(nodes + 4 * w.cur + 0);
        const float4 n1 = __ldg(nodes + 4 * w.cur + 1);
        const float4 n2 = __ldg(nodes + 4 * w.cur + 2);
        const float4 n3 = __ldg(nodes + 4 * w.cur + 3);
        const float tmax = walk_cull<false>(w);
        float ta, tb;
        const bool h0 = ray_aabb(n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, ox, oy, oz, w.ix, w.iy, w.iz, tmax, ta);
        const bool h1 = ray_aabb(n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, ox, oy, oz, w.ix, w.iy, w.iz, tmax, tb);
        const int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
        if (h0 && h1) {
          int nr, fr;
          float nt, ft;
          if (ta <= tb) { nr = c0; nt = ta; fr = c1; ft = tb; }
          else { nr = c1; nt = tb; fr = c0; ft = ta; }
          if (w.sp < STACK_DEPTH) {
            w.stack_ref[w.sp] = fr;
            w.stack_t[w.sp] = ft;
            w.sp++;
          } else {
            atomicOr(err, 1u);
          }
          w.cur = (walk_have(w) && nt >= w.t_best) ? walk_pop<TIE>(w) : nr;
        } else if (h0) {
          w.cur = (walk_have(w) && ta >= w.t_best) ? walk_pop<TIE>(w) : c0;
        } else if (h1) {
          w.cur = (walk_have(w) && tb >= w.t_best) ? walk_pop<TIE>(w) : c1;
        } else {
          w.cur = walk_pop<TIE>(w);
        }
      } else {
        bool have = walk_have(w);
        float t_cull = walk_cull<false>(w);
        uint32_t sb = 0, tb = 0;
        TieState ts = tie_begin();
        leaf_test<false>(prims, w.cur, ox, oy, oz, dx, dy, dz, have, w.t_best, t_cull, w.prim_best, sb, tb, ts);
        w.cur = walk_pop<TIE>(w);
      }
    }
    return w.cur == kDone;
  }
  return walk_spec(w, S, ox, oy, oz, dx, dy, dz, steps, err);
}

// A ray parked between two segments: its state into the per-ray records, for
// the next epoch to restore. (Out of line, as the epoch bookkeeping below: a
// single-launch trace never runs them, and the persistent loop stays small
// enough for the instruction cache.)
template <int NB>
__device__ __noinline__ void park_ray(const WfState& rs, uint32_t rid, float px, float py, float pz, float dist,
                                      float dx, float dy, float dz, uint32_t rng_s, Bands<NB> e, uint32_t bounce) {
  rs.pos[rid] = make_float4(px, py, pz, dist);
  rs.dir[rid] = make_float4(dx, dy, dz, __uint_as_float(rng_s));
  float v[8];
#pragma unroll
  for (int b = 0; b < 8; b++) v[b] = b < NB ? e.v[b] : 0.0f;
  rs.e[rid] = make_float4(v[0], v[1], v[2], v[3]);
  if (NB > 4) rs.e[rs.cap + rid] = make_float4(v[4], v[5], v[6], v[7]);
  rs.bounce[rid] = bounce;
}

// An epoch's per-iteration bookkeeping, warp-aggregated (every lane calls it):
// count the ended rays (and raise the park signal once at most `keep` remain
// and the queue is drained), append the parked ones to the next epoch's queue.
__device__ __noinline__ void epoch_tally(const EpochArgs& ea, bool ended, bool parked, uint32_t rid, bool may_park,
                                         uint32_t n_rays, uint32_t keep, const uint32_t* fetch) {
  const unsigned FULL = 0xffffffffu;
  const uint32_t lane = threadIdx.x & 31u, lt_mask = (1u << lane) - 1u;
  const unsigned em = __ballot_sync(FULL, ended);
  if (em && lane == (uint32_t)(__ffs(em) - 1)) {
    const uint32_t done_now = atomicAdd(&ea.cur->ended, (uint32_t)__popc(em)) + (uint32_t)__popc(em);
    if (may_park && n_rays - done_now <= keep && *((volatile const uint32_t*)fetch) >= n_rays)
      *((volatile uint32_t*)&ea.cur->park) = 1u;
  }
  const unsigned pm = __ballot_sync(FULL, parked);
  if (pm) {
    uint32_t base = 0;
    if (lane == (uint32_t)(__ffs(pm) - 1)) base = atomicAdd(&ea.next->n, (uint32_t)__popc(pm));
    base = __shfl_sync(FULL, base, __ffs(pm) - 1);
    if (parked) ea.out_q[base + (uint32_t)__popc(pm & lt_mask)] = rid;
  }
}

// The tracer. Each lane runs a small state machine so that a lane whose
// closest-hit walk ends shades its segment and starts the next one at once,
// while the other lanes of its warp keep walking: per loop iteration a lane
// takes at most `walk_steps` traversal steps, then shades if its walk is done.
// Idle lanes refill from the global ray queue. Walking and shading alternate
// per warp: lanes whose walk is done wait until `shade_min` of them can shade
// together (or nothing else is walking), so the shading code, which is long,
// does not run once per lane.
//
// In an epoch chain (ea.cur set) the queue is this epoch's: fresh rays, or
// parked rays whose state is restored from the per-ray records. Once at most
// park_pct % of the epoch's rays remain and its queue is drained, each lane
// parks its ray at the end of its current segment, so that the next epoch
// runs the survivors in full warps. An epoch whose park signal is never
// raised (it ended too few rays while rays were still queued) runs its rays
// to their end, which is only slower.
//
// WIDE (near-tie rule only): walks on the 4-wide tree. A template parameter,
// not a runtime flag, so that each variant carries only its own walk: the
// loop body is then small enough for the instruction cache.
//
// Registers: the launch bound (256, 4) caps a thread at 64. Across the loop a
// lane keeps only what the walk reads (the ray, its job, the walk state); the
// segment's hit is computed in the shading pass from the walk's result, and
// the state that only the refill and the shading pass touch (energies,
// distance, stream, segment count, ray id) lives, for up to 4 bands, in shared
// memory, a column per thread. The 3-band near-tie kernel then has 16 bytes of
// spill stores, against 184 with that state in registers.
template <int NB, bool TIE, bool WIDE, bool WT>
__global__ void __launch_bounds__(256, 4) trace_kernel(const DJob* __restrict__ jobs, uint32_t n_jobs,
                                                       uint32_t total_rays, const DScene* __restrict__ scenes,
                                                       const DMat* __restrict__ job_mats,
                                                       const DPanel* __restrict__ panels,
                                                       const DPanelGroup* __restrict__ groups, float* __restrict__ acc,
                                                    DLaunch* __restrict__ hdr, uint32_t* __restrict__ job_segments,
                                                    uint32_t refill_min, int walk_budget, uint32_t shade_min,
                                                    EpochArgs ea) {
  constexpr bool wide = TIE && WIDE;
  const unsigned FULL = 0xffffffffu;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lt_mask = (1u << lane) - 1u;
  enum { IDLE = 0, WALK = 1, SHADE = 2 };
  int phase = IDLE;
  bool exhausted = false;
  uint32_t ji = 0;
  float px = 0, py = 0, pz = 0, dx = 0, dy = 0, dz = 0;
  // the ray's state that only the refill and the shading pass touch
  // (energies, distance travelled, stream, segments so far, ray id): for up to
  // 4 bands a column per thread in shared memory, so that it holds no
  // registers across the walk; for 8 bands in registers (there the shared
  // copy's loads and stores in every shading pass cost more than it saves)
  constexpr bool kColdShared = NB <= 4;
  constexpr int kCols = kColdShared ? kMaxWarps * 32 : 1;
  __shared__ float s_e[kColdShared ? NB : 1][kCols];
  __shared__ float s_dist[kCols];
  __shared__ uint32_t s_rng[kCols], s_bounce[kCols], s_rid[kCols];
  const uint32_t me = kColdShared ? threadIdx.x : 0u;
  float r_e[NB];
  float r_dist = 0.0f;
  uint32_t r_rng = 0, r_bounce = 0, r_rid = 0;
  auto cold_save = [&](const float* ev, float dist, uint32_t rng_s, uint32_t bounce) {
#pragma unroll
    for (int b = 0; b < NB; b++) {
      if constexpr (kColdShared) s_e[b][me] = ev[b];
      else r_e[b] = ev[b];
    }
    if constexpr (kColdShared) {
      s_dist[me] = dist;
      s_rng[me] = rng_s;
      s_bounce[me] = bounce;
    } else {
      r_dist = dist;
      r_rng = rng_s;
      r_bounce = bounce;
    }
  };
  auto cold_load = [&](float* ev, float& dist, uint32_t& rng_s, uint32_t& bounce) {
#pragma unroll
    for (int b = 0; b < NB; b++) ev[b] = kColdShared ? s_e[b][me] : r_e[b];
    dist = kColdShared ? s_dist[me] : r_dist;
    rng_s = kColdShared ? s_rng[me] : r_rng;
    bounce = kColdShared ? s_bounce[me] : r_bounce;
  };
  auto cold_set_rid = [&](uint32_t rid) {
    if constexpr (kColdShared) s_rid[me] = rid;
    else r_rid = rid;
  };
  auto cold_rid = [&]() { return kColdShared ? s_rid[me] : r_rid; };
  int walk_stack_ref[STACK_DEPTH];
  float walk_stack_t[STACK_DEPTH];
  Walk w;
  w.stack_ref = walk_stack_ref;
  w.stack_t = walk_stack_t;
  uint32_t* err = &hdr->error;
  const WfState& rs = ea.st;
  const uint32_t* rq = ea.in_q;
  const uint32_t n_rays = ea.cur ? (rq ? ea.cur->n : total_rays) : total_rays;
  uint32_t* fetch = ea.cur ? &ea.cur->fetch : &hdr->ray_counter;
  const bool may_park = ea.cur && ea.out_q && n_rays > ea.park_min;
  const uint32_t keep = (uint32_t)(((uint64_t)n_rays * ea.park_pct) / 100u);
  bool parking = false;
  uint32_t iters = 0;   // loop guard (warp-uniform: every lane runs every iteration)
  __shared__ uint8_t s_slots[kMaxWarps][256];   // coop_leaf_rounds' slot lists, one per warp

  // begin one segment from (p, d): a mesh walk, or (a shoebox) the shading
  // pass at once, which computes the box hit
  auto begin_segment = [&](const DJob& J) {
    if (J.geom == OMG_GEOM_BOX) {
      phase = SHADE;
    } else {
      walk_begin<TIE>(w, scenes[J.scene], px, py, pz, dx, dy, dz, wide);
      phase = WALK;
    }
  };

  while (true) {
    if (++iters > ea.max_loop) {
      atomicOr(err, 8u);
      break;
    }
    // ---- refill idle lanes from the ray queue (warp-aggregated)
    const unsigned idle = __ballot_sync(FULL, phase == IDLE);
    if (!exhausted && idle != 0u && (__popc(idle) >= (int)refill_min || idle == FULL)) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(fetch, (uint32_t)__popc(idle));
      base = __shfl_sync(FULL, base, 0);
      if (base >= n_rays) exhausted = true;
      if (phase == IDLE) {
        const uint32_t k = base + (uint32_t)__popc(idle & lt_mask);
        if (k < n_rays) {
          if (rq) {
            const uint32_t rid = rq[k];
            ji = find_job(jobs, n_jobs, rid);
            const float4 P = rs.pos[rid], D = rs.dir[rid];
            px = P.x; py = P.y; pz = P.z;
            dx = D.x; dy = D.y; dz = D.z;
            const float4 e0 = rs.e[rid];
            const float4 e1 = NB > 4 ? rs.e[rs.cap + rid] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            const float ev[8] = {e0.x, e0.y, e0.z, e0.w, e1.x, e1.y, e1.z, e1.w};
            cold_save(ev, P.w, __float_as_uint(D.w), rs.bounce[rid]);
            cold_set_rid(rid);
          } else {
            const uint32_t rid = k;
            ji = find_job(jobs, n_jobs, rid);
            const DJob& J = jobs[ji];
            Pcg rng;
            rng.init(J.seed, rid - J.ray_base);
            unit_sphere(rng, dx, dy, dz);
            px = J.src[0]; py = J.src[1]; pz = J.src[2];
            cold_save(J.e0, 0.0f, rng.s, 0u);
            cold_set_rid(rid);
          }
          begin_segment(jobs[ji]);
        }
      }
    }
    if (__ballot_sync(FULL, phase != IDLE) == 0u) {
      if (exhausted) break;
      continue;
    }
    // the epoch's park signal (sticky; raised only once its queue is drained)
    if (may_park && !parking) parking = *((volatile const uint32_t*)&ea.cur->park) != 0u;

    // ---- this iteration either shades or walks, for the whole warp: lanes
    // whose walk is done wait until at least shade_min of them are ready (or
    // no lane is walking), so that the shading code runs with full lanes
    const unsigned walking = __ballot_sync(FULL, phase == WALK);
    const unsigned ready = __ballot_sync(FULL, phase == SHADE);
    const bool shade_now = ready != 0u && (walking == 0u || __popc(ready) >= (int)shade_min);

    // ---- closest-hit walk, at most walk_budget steps this iteration; a lane
    // whose walk is over waits to shade, its result kept in w until then
    if (TIE && !wide) {
      // near-tie walks on the binary tree: the node phase lane by lane, then
      // the pending leaves tested by the whole warp together
      if (!shade_now) {
        const bool wk = phase == WALK;
        const float4* lp = nullptr;
        bool over = false, lwt = false;
        if (wk) {
          const DScene& S = scenes[jobs[ji].scene];
          lwt = WT && S.prims_wt != nullptr;
          lp = lwt ? S.prims_wt : S.prims;
          int st = walk_budget;
          over = walk_spec_nodes(w, S, px, py, pz, dx, dy, dz, st, err);
        }
        coop_leaf_rounds<WT>(w, wk && !over, lp, lwt, px, py, pz, dx, dy, dz, s_slots[threadIdx.x >> 5],
                             kCoopRounds, err);
        if (wk) {
          const DScene& S = scenes[jobs[ji].scene];
          // an ambiguous near-tie window: the walk starts over in fixed mode
          if (!over && w.cur == kDone && w.leaf == 0) over = !walk_restart_fixed(w, S.root, S.walk_budget);
          if (over) phase = SHADE;
        }
      }
    } else if (!shade_now && phase == WALK) {
      const DJob& J = jobs[ji];
      const DScene& S = scenes[J.scene];
      if (walk_steps<TIE>(w, S, px, py, pz, dx, dy, dz, walk_budget, wide, err)) phase = SHADE;
    }

    // ---- one segment of the bounce loop (tracer.rs:103-200)
    bool ended = false, parked = false;
    if (shade_now && phase == SHADE) {
      const DJob& J = jobs[ji];
      // the segment's closest hit: the shoebox's, or the walk's (normal of
      // the original triangle, against d)
      Hit h;
      h.t = FLT_MAX;
      h.m = nullptr;
      bool have;
      if (J.geom == OMG_GEOM_BOX) {
        have = box_hit(J, job_mats, px, py, pz, dx, dy, dz, h);
      } else {
        const DScene& S = scenes[J.scene];
        have = walk_have(w);
        if (have) {
          const float4 p0 = __ldg(S.prims + 3 * w.prim_best + 0);
          const float4 p1 = __ldg(S.prims + 3 * w.prim_best + 1);
          const float4 nn = __ldg(S.normals + __float_as_uint(p1.w));
          float nx = nn.x, ny = nn.y, nz = nn.z;
          if (nx * dx + ny * dy + nz * dz > 0.0f) { nx = nx * -1.0f; ny = ny * -1.0f; nz = nz * -1.0f; }
          h.t = w.t_best;
          h.nx = nx; h.ny = ny; h.nz = nz;
          h.m = S.mats + __float_as_uint(p0.w);
        }
      }
      if (J.n_groups) have = panels_hit(J, panels, groups, job_mats, px, py, pz, dx, dy, dz, have, h);
      const float t_hit = have ? h.t : FLT_MAX;
      float e[NB], dist;
      Pcg rng;
      uint32_t bounce;
      cold_load(e, dist, rng.s, bounce);
      bool done = shade_segment<NB>(J, acc, h, have, t_hit, px, py, pz, dx, dy, dz, dist, e, rng);
      bounce++;
      if (!done && bounce >= J.max_bounces) done = true;
      if (done) {
        atomicAdd(job_segments + ji, bounce);
        phase = IDLE;
        ended = true;
      } else if (parking) {
        // save the ray between two segments; the next epoch restores it
        Bands<NB> eb;
#pragma unroll
        for (int b = 0; b < NB; b++) eb.v[b] = e[b];
        park_ray<NB>(rs, cold_rid(), px, py, pz, dist, dx, dy, dz, rng.s, eb, bounce);
        phase = IDLE;
        parked = true;
      } else {
        cold_save(e, dist, rng.s, bounce);
        begin_segment(J);
      }
    }
    if (ea.cur) epoch_tally(ea, ended, parked, cold_rid(), may_park, n_rays, keep, fetch);
  }
}

// The tracer as a wavefront inside each warp. A lane walks one ray at a time;
// when its walk ends, the ray id goes to the warp's shading queue and the lane
// takes the next ray to walk from the warp's walk queue (or the global ray
// queue). Once shade_min rays wait in the shading queue (32 by default; or
// nothing is left to walk) the whole warp shades up to 32 of them together,
// from their saved state, and the survivors join the walk queue. Walks thus
// refill lane by lane, and the long shading code runs with full warps (a
// smaller shade_min trades that for shorter waits when few rays are left). A
// warp owns at most 63 rays
// between two fetches from the ray queue (fetching only once its walk queue
// is empty, with at most 31 waiting for shading and 32 walking), so each
// queue holds 64 ids.
//
// Epochs (ea.cur set) work as in trace_kernel: once parking, survivors of a
// shading pass and rays waiting to walk go to the next epoch's queue.
template <int NB, bool TIE>
__global__ void __launch_bounds__(256, 4) trace_wl_kernel(const DJob* __restrict__ jobs, uint32_t n_jobs,
                                                          uint32_t total_rays, const DScene* __restrict__ scenes,
                                                          const DMat* __restrict__ job_mats,
                                                          const DPanel* __restrict__ panels,
                                                          const DPanelGroup* __restrict__ groups,
                                                          float* __restrict__ acc, DLaunch* __restrict__ hdr,
                                                          uint32_t* __restrict__ job_segments, int walk_budget,
                                                          uint32_t shade_min, bool wide, EpochArgs ea) {
  constexpr unsigned FULL = 0xffffffffu;
  constexpr uint32_t kNone = 0xFFFFFFFFu;
  constexpr uint32_t kQ = 64;
  __shared__ uint32_t s_shade[8][kQ];
  __shared__ uint32_t s_walk[8][kQ];
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lt_mask = (1u << lane) - 1u;
  uint32_t* shade_q = s_shade[threadIdx.x >> 5];
  uint32_t* walk_q = s_walk[threadIdx.x >> 5];
  uint32_t sh_head = 0, sh_cnt = 0, wk_head = 0, wk_cnt = 0;   // warp-uniform
  const WfState& st = ea.st;
  const uint32_t* rq = ea.in_q;
  const uint32_t n_rays = ea.cur ? (rq ? ea.cur->n : total_rays) : total_rays;
  uint32_t* fetch = ea.cur ? &ea.cur->fetch : &hdr->ray_counter;
  const bool may_park = ea.cur && ea.out_q && n_rays > ea.park_min;
  const uint32_t keep = (uint32_t)(((uint64_t)n_rays * ea.park_pct) / 100u);
  bool parking = false, exhausted = false;
  uint32_t* err = &hdr->error;

  // the walking ray of this lane
  uint32_t rid = kNone;
  const DScene* wsc = nullptr;
  float ox = 0, oy = 0, oz = 0, dx = 0, dy = 0, dz = 0;
  int walk_stack_ref[STACK_DEPTH];
  float walk_stack_t[STACK_DEPTH];
  Walk w;
  w.stack_ref = walk_stack_ref;
  w.stack_t = walk_stack_t;

  auto start_walk = [&](uint32_t r) {
    const DJob& J = jobs[find_job(jobs, n_jobs, r)];
    const float4 P = st.pos[r], D = st.dir[r];
    ox = P.x; oy = P.y; oz = P.z;
    dx = D.x; dy = D.y; dz = D.z;
    wsc = scenes + J.scene;
    walk_begin<TIE>(w, *wsc, ox, oy, oz, dx, dy, dz, wide);
    rid = r;
  };
  // ended rays (and the park signal), parked rays to the next epoch's queue
  auto epoch_tally = [&](bool ended, bool parked, uint32_t r) {
    if (!ea.cur) return;
    const unsigned em = __ballot_sync(FULL, ended);
    if (em && lane == (uint32_t)(__ffs(em) - 1)) {
      const uint32_t done_now = atomicAdd(&ea.cur->ended, (uint32_t)__popc(em)) + (uint32_t)__popc(em);
      if (may_park && n_rays - done_now <= keep && *((volatile const uint32_t*)fetch) >= n_rays)
        *((volatile uint32_t*)&ea.cur->park) = 1u;
    }
    const unsigned pm = __ballot_sync(FULL, parked);
    if (pm) {
      uint32_t base = 0;
      if (lane == (uint32_t)(__ffs(pm) - 1)) base = atomicAdd(&ea.next->n, (uint32_t)__popc(pm));
      base = __shfl_sync(FULL, base, __ffs(pm) - 1);
      if (parked) ea.out_q[base + (uint32_t)__popc(pm & lt_mask)] = r;
    }
  };

  uint32_t iters = 0;   // loop guard (warp-uniform)
  while (true) {
    if (++iters > ea.max_loop) {
      atomicOr(err, 8u);
      break;
    }
    if (may_park && !parking) parking = *((volatile const uint32_t*)&ea.cur->park) != 0u;
    if (parking && wk_cnt) {
      // rays waiting to walk are between two segments: park them as they are
      const uint32_t m = wk_cnt < 32u ? wk_cnt : 32u;
      const bool pk = lane < m;
      const uint32_t r = pk ? walk_q[(wk_head + lane) % kQ] : kNone;
      wk_head += m;
      wk_cnt -= m;
      epoch_tally(false, pk, r);
      __syncwarp();
      continue;
    }
    unsigned walking = __ballot_sync(FULL, rid != kNone);

    // ---- shading pass: a full warp of rays, or whatever waits once nothing can walk
    if (sh_cnt >= shade_min || (sh_cnt && !walking && !wk_cnt && (exhausted || parking))) {
      const uint32_t m = sh_cnt < 32u ? sh_cnt : 32u;
      bool alive = false, ended = false;
      uint32_t r = kNone;
      if (lane < m) {
        r = shade_q[(sh_head + lane) % kQ];
        alive = shade_saved_ray<NB>(jobs, n_jobs, scenes, job_mats, panels, groups, acc, st, r, job_segments);
        ended = !alive;
      }
      sh_head += m;
      sh_cnt -= m;
      const bool parked = alive && parking;
      alive = alive && !parking;
      const unsigned am = __ballot_sync(FULL, alive);
      if (alive) walk_q[(wk_head + wk_cnt + (uint32_t)__popc(am & lt_mask)) % kQ] = r;
      wk_cnt += (uint32_t)__popc(am);
      epoch_tally(ended, parked, r);
      __syncwarp();
      continue;
    }

    // ---- idle lanes take rays: the walk queue first, then the ray queue
    unsigned idle = ~walking;
    if (idle && wk_cnt) {
      const uint32_t rank = (uint32_t)__popc(idle & lt_mask);
      const uint32_t k = (uint32_t)__popc(idle) < wk_cnt ? (uint32_t)__popc(idle) : wk_cnt;
      if (rid == kNone && rank < k) start_walk(walk_q[(wk_head + rank) % kQ]);
      wk_head += k;
      wk_cnt -= k;
      idle = __ballot_sync(FULL, rid == kNone);
    }
    if (idle && !wk_cnt && !exhausted && !parking) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(fetch, (uint32_t)__popc(idle));
      base = __shfl_sync(FULL, base, 0);
      if (base >= n_rays) exhausted = true;
      bool to_shade = false;
      uint32_t r = kNone;
      if (rid == kNone) {
        const uint32_t k = base + (uint32_t)__popc(idle & lt_mask);
        if (k < n_rays) {
          r = rq ? rq[k] : k;
          const DJob& J = jobs[find_job(jobs, n_jobs, r)];
          if (!rq) start_saved_ray<NB>(J, st, r);
          // a shoebox needs no walk: its hit is found when the ray is shaded
          if (J.geom == OMG_GEOM_BOX) to_shade = true;
          else start_walk(r);
        }
      }
      const unsigned bm = __ballot_sync(FULL, to_shade);
      if (to_shade) shade_q[(sh_head + sh_cnt + (uint32_t)__popc(bm & lt_mask)) % kQ] = r;
      sh_cnt += (uint32_t)__popc(bm);
    }
    walking = __ballot_sync(FULL, rid != kNone);
    if (!walking && !sh_cnt && !wk_cnt && (exhausted || parking)) break;

    // ---- walk, at most walk_budget steps this iteration
    bool finished = false;
    if (rid != kNone && walk_steps<TIE>(w, *wsc, ox, oy, oz, dx, dy, dz, walk_budget, wide, err)) {
      st.hit[rid] = make_float2(w.t_best, __int_as_float(w.prim_best));
      finished = true;
    }
    const unsigned fm = __ballot_sync(FULL, finished);
    if (finished) {
      shade_q[(sh_head + sh_cnt + (uint32_t)__popc(fm & lt_mask)) % kQ] = rid;
      rid = kNone;
    }
    sh_cnt += (uint32_t)__popc(fm);
    __syncwarp();
  }
}

// out = (sum + comp) * 2^-64 per float, bins then dirs, per job.
__global__ void finalize_kernel(const DJob* __restrict__ jobs, uint32_t n_jobs, const float* __restrict__ acc,
                                float* __restrict__ out) {
  const uint32_t j = blockIdx.y;
  if (j >= n_jobs) return;
  const DJob& J = jobs[j];
  const uint32_t nbb = J.n_bins * J.nb, nd = J.n_bins * 3;
  const float* A = acc + J.acc_off;
  float* O = out + J.out_off;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nbb + nd; i += gridDim.x * blockDim.x) {
    float v;
    if (i < nbb) v = A[i] + A[nbb + i];
    else v = A[2 * nbb + (i - nbb)] + A[2 * nbb + nd + (i - nbb)];
    O[i] = v * kAccUnscale;
  }
}

template <bool TIE>
__global__ void raycast_kernel(const DScene* __restrict__ scene, const float* __restrict__ o,
                               const float* __restrict__ d, uint32_t n, float* __restrict__ t_out,
                               uint32_t* __restrict__ tri_out, DLaunch* hdr) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const DScene S = *scene;
  float t;
  int prim = 0;
  const float ox = o[3 * i], oy = o[3 * i + 1], oz = o[3 * i + 2];
  const float dx = d[3 * i], dy = d[3 * i + 1], dz = d[3 * i + 2];
  bool have = (TIE && S.nodes4) ? mesh_closest4(S, ox, oy, oz, dx, dy, dz, t, prim, &hdr->error)
                                : mesh_closest<TIE>(S, ox, oy, oz, dx, dy, dz, t, prim, &hdr->error);
  if (have) {
    t_out[i] = t;
    tri_out[i] = __float_as_uint(__ldg(S.prims + 3 * prim + 1).w);
  } else {
    t_out[i] = -1.0f;
    tri_out[i] = 0xFFFFFFFFu;
  }
}

}  // namespace

cudaError_t launch_trace(const DJob* jobs, uint32_t n_jobs, uint32_t total_rays, uint32_t max_nb,
                         const DScene* scenes, const DMat* job_mats, const DPanel* panels,
                         const DPanelGroup* groups, float* acc, DLaunch* hdr,
                         uint32_t* job_segments, const LaunchShape& shape, int n_sms, bool tie, cudaStream_t s,
                         const EpochArgs* ep, bool wt) {
  if (n_jobs == 0 || total_rays == 0) return cudaSuccess;
  EpochArgs ea{};
  if (ep) ea = *ep;
  // loop iterations of one warp of a persistent kernel before it gives up and
  // flags error 8: by default far above any legitimate count (each iteration
  // advances a walk, a shading pass or the ray queue)
  ea.max_loop = shape.loop_guard ? shape.loop_guard : kDefaultLoopGuard;
  if (shape.mode == 2 && tie && ea.st.pos)
    return launch_trace_coop(jobs, n_jobs, total_rays, max_nb, scenes, job_mats, panels, groups, acc, hdr,
                             job_segments, shape, n_sms, ea, s);
  uint32_t threads = shape.block_threads;
  uint64_t want = (uint64_t)n_sms * shape.blocks_per_sm;
  uint64_t need = ((uint64_t)total_rays + threads - 1) / threads;
  uint32_t blocks = (uint32_t)(want < need ? want : need);
  if (blocks == 0) blocks = 1;
  uint32_t refill = shape.refill_min == 0 ? 1 : (shape.refill_min > 32 ? 32 : shape.refill_min);
  const int steps = shape.walk_steps == 0 ? 1000000 : (int)shape.walk_steps;
  const uint32_t shade_min = shape.shade_min == 0 ? 1u : (shape.shade_min > 32 ? 32u : shape.shade_min);
  // the warp-local wavefront needs the per-ray records and at most 8 warps a block
  const bool wl = shape.mode == 1 && ea.st.pos && threads <= 256;
  const uint32_t wl_shade = shape.wl_shade_min == 0 ? 32u : (shape.wl_shade_min > 32 ? 32u : shape.wl_shade_min);
  const bool wide = shape.wide != 0;
#define OMG_TRACE_LAUNCH(NB, TIE)                                                                         \
  if (wl)                                                                                                      \
    trace_wl_kernel<NB, TIE><<<blocks, threads, 0, s>>>(jobs, n_jobs, total_rays, scenes, job_mats, panels,    \
                                                        groups, acc, hdr, job_segments, steps, wl_shade, wide, ea);  \
  else if (TIE && wide)                                                                                        \
    trace_kernel<NB, TIE, true, false><<<blocks, threads, 0, s>>>(jobs, n_jobs, total_rays, scenes, job_mats,   \
                                                                  panels, groups, acc, hdr, job_segments, refill, \
                                                                  steps, shade_min, ea);                          \
  else if (TIE && wt)                                                                                          \
    trace_kernel<NB, TIE, false, true><<<blocks, threads, 0, s>>>(jobs, n_jobs, total_rays, scenes, job_mats,   \
                                                                  panels, groups, acc, hdr, job_segments, refill, \
                                                                  steps, shade_min, ea);                          \
  else                                                                                                         \
    trace_kernel<NB, TIE, false, false><<<blocks, threads, 0, s>>>(jobs, n_jobs, total_rays, scenes, job_mats,  \
                                                                   panels, groups, acc, hdr, job_segments, refill,\
                                                                   steps, shade_min, ea)
  if (max_nb <= 3) {
    if (tie) OMG_TRACE_LAUNCH(3, true);
    else OMG_TRACE_LAUNCH(3, false);
  } else {
    if (tie) OMG_TRACE_LAUNCH(8, true);
    else OMG_TRACE_LAUNCH(8, false);
  }
#undef OMG_TRACE_LAUNCH
  return cudaGetLastError();
}

cudaError_t preload_trace_kernels() {
  cudaFuncAttributes fa;
  cudaError_t e;
  if ((e = cudaFuncGetAttributes(&fa, trace_kernel<3, false, false, false>)) != cudaSuccess) return e;
  if ((e = cudaFuncGetAttributes(&fa, trace_kernel<3, true, false, false>)) != cudaSuccess) return e;
  if ((e = cudaFuncGetAttributes(&fa, trace_kernel<8, false, false, false>)) != cudaSuccess) return e;
  return cudaFuncGetAttributes(&fa, trace_kernel<8, true, false, false>);
}

cudaError_t launch_finalize(const DJob* jobs, uint32_t n_jobs, const float* acc, float* out, uint64_t total_out,
                            cudaStream_t s) {
  if (n_jobs == 0) return cudaSuccess;
  (void)total_out;
  dim3 grid(8, n_jobs);
  finalize_kernel<<<grid, 256, 0, s>>>(jobs, n_jobs, acc, out);
  return cudaGetLastError();
}

cudaError_t launch_raycast(const DScene* scene, const float* o, const float* d, uint32_t n, float* t, uint32_t* tri,
                           DLaunch* hdr, bool tie, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  if (tie) raycast_kernel<true><<<(n + 127) / 128, 128, 0, s>>>(scene, o, d, n, t, tri, hdr);
  else raycast_kernel<false><<<(n + 127) / 128, 128, 0, s>>>(scene, o, d, n, t, tri, hdr);
  return cudaGetLastError();
}

}  // namespace omg
