// Persistent tracer with cooperative walks (launch shape mode 2).
//
// Each closest-hit walk is split over a group of 4 lanes: one lane per child
// of the 4-wide tree (DScene::nodes4c), so a node step is one child-box test
// per lane, the lanes of a hit leaf test its primitives, a 2-step shuffle
// reduction applies the near-tie rule, and the group descends into its
// nearest internal child, pushing the others (farthest first) onto the
// group's stack in shared memory. A warp walks 8 rays at once in full lockstep
// of its 32 lanes; a group whose walk ends hands the ray id to the warp's
// shading queue and takes the next ray from the warp's walk queue (or the
// global ray queue). Shading runs one ray per lane, 32 rays at a time, from
// the saved per-ray state (shade_saved_ray), as in the warp-local wavefront
// kernel (trace.cu).
//
// The near-tie rule (tie_mode 1) makes the winning triangle independent of
// the visit order, so walks in any order find the hit the reference's walk
// finds, up to chains of near-ties; boxes are skipped only beyond
// best * (1 + 1e-6). Everything else follows the reference's bounce loop
// (tracer.rs:103-200) operation by operation.
#include "shade_common.cuh"

namespace omg {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kQ = 64;                 // warp queues (at most 8 + 31 + 32 rays owned, see below)
constexpr int kDoneC = 0x7FFFFFFF;
constexpr int kGroupsPerBlock = 64;         // 256 threads / 4

// Two lanes' near-tie states merged (TieState, device_common.cuh): the union
// of the hits both have seen. The nearer t_min sets the window; a winner
// outside it drops out, and if its lane had seen hits inside the window that
// it no longer knows, the merged state is ambiguous. Winners compare by
// (surface, triangle, t, primitive), a total order, so every lane of a group
// reduces to the same state. In fixed mode the window is final and only the
// lowest key counts.
__device__ __forceinline__ void tie_merge(bool& ah, float& at, uint32_t& as, uint32_t& atr, int& ap, float& amin,
                                          bool& aamb, bool bh, float bt, uint32_t bs, uint32_t btr, int bp,
                                          float bmin, bool bamb, bool fixed) {
  if (!bh) return;
  bool take_b;
  if (!ah) {
    take_b = true;
    amin = bmin;
    aamb = bamb;
  } else {
    const bool b_less = tie_key_less(bs, btr, bt, as, atr, at) || (bs == as && btr == atr && bt == at && bp < ap);
    if (fixed) {
      take_b = b_less;
    } else {
      const float tmin = fminf(amin, bmin);
      const float win = tmin * (1.0f + kTieRel);
      const bool ain = at <= win, bin = bt <= win;
      aamb = aamb || bamb || (!ain && amin <= win) || (!bin && bmin <= win);
      take_b = (ain && bin) ? b_less : bin;
      amin = tmin;
    }
  }
  if (take_b) {
    ah = true;
    at = bt;
    as = bs;
    atr = btr;
    ap = bp;
  }
}

template <int NB>
__global__ void __launch_bounds__(256, 4) trace_coop_kernel(const DJob* __restrict__ jobs, uint32_t n_jobs,
                                                            uint32_t total_rays, const DScene* __restrict__ scenes,
                                                            const DMat* __restrict__ job_mats,
                                                            const DPanel* __restrict__ panels,
                                                            const DPanelGroup* __restrict__ groups,
                                                            float* __restrict__ acc, DLaunch* __restrict__ hdr,
                                                            uint32_t* __restrict__ job_segments, int walk_budget,
                                                            uint32_t shade_min, EpochArgs ea) {
  __shared__ uint32_t s_shade[8][kQ];
  __shared__ uint32_t s_walk[8][kQ];
  __shared__ int s_sref[kGroupsPerBlock][STACK_DEPTH];
  __shared__ float s_st[kGroupsPerBlock][STACK_DEPTH];
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const uint32_t sub = lane & 3u;           // the child this lane tests
  const uint32_t gbase = lane & ~3u;        // first lane of the group
  const bool leader = sub == 0u;
  int* sref = s_sref[threadIdx.x >> 2];
  float* sst = s_st[threadIdx.x >> 2];
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

  // the group's walk (the same values in its 4 lanes)
  uint32_t rid = kNone;
  const float4* nodes = nullptr;
  const float4* prims = nullptr;
  bool pwt = false;   // watertight context: prims holds the exact vertices
  float ox = 0, oy = 0, oz = 0, dx = 0, dy = 0, dz = 0, ix = 0, iy = 0, iz = 0;
  int cur = kDoneC, sp = 0;
  bool have = false;
  float t_best = FLT_MAX, t_cull = FLT_MAX;
  uint32_t s_best = 0, tri_best = 0, budget = 0, budget0 = 0;
  int prim_best = -1, root = kDoneC;
  TieState ts = tie_begin();

  auto start_walk = [&](uint32_t r) {
    const DJob& J = jobs[find_job(jobs, n_jobs, r)];
    const float4 P = st.pos[r], D = st.dir[r];
    ox = P.x; oy = P.y; oz = P.z;
    dx = D.x; dy = D.y; dz = D.z;
    ix = __frcp_rn(dx); iy = __frcp_rn(dy); iz = __frcp_rn(dz);
    const DScene& S = scenes[J.scene];
    nodes = S.nodes4c;
    pwt = S.prims_wt != nullptr;
    prims = pwt ? S.prims_wt : S.prims;
    // a shoebox ray (its hit is found when it is shaded) or an empty scene:
    // the walk ends at its first step without reading a node
    const bool walkable = J.geom == OMG_GEOM_MESH && S.n_prims != 0u && nodes != nullptr;
    cur = walkable ? S.root4 : kDoneC;
    root = cur;
    budget0 = walkable ? S.walk_budget4 : 1u;   // every node is entered at most once per pass
    budget = budget0;
    sp = 0;
    have = false;
    t_best = FLT_MAX;
    t_cull = FLT_MAX;
    s_best = 0;
    tri_best = 0;
    prim_best = -1;
    ts = tie_begin();
    rid = r;
  };
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

  uint32_t iters = 0;
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
    unsigned walking = __ballot_sync(FULL, leader && rid != kNone);

    // ---- shading pass, one ray per lane: once shade_min rays wait (at most 32 shade together), or
    // whatever waits once nothing can walk
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

    // ---- idle groups take rays: the walk queue first, then the ray queue
    unsigned idle = __ballot_sync(FULL, leader && rid == kNone);
    if (idle && wk_cnt) {
      const uint32_t n_idle = (uint32_t)__popc(idle);
      const uint32_t k = n_idle < wk_cnt ? n_idle : wk_cnt;
      uint32_t r = kNone;
      if (leader && rid == kNone) {
        const uint32_t rank = (uint32_t)__popc(idle & lt_mask);
        if (rank < k) r = walk_q[(wk_head + rank) % kQ];
      }
      r = __shfl_sync(FULL, r, gbase);
      if (r != kNone) start_walk(r);
      wk_head += k;
      wk_cnt -= k;
      idle = __ballot_sync(FULL, leader && rid == kNone);
    }
    if (idle && !wk_cnt && !exhausted && !parking) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(fetch, (uint32_t)__popc(idle));
      base = __shfl_sync(FULL, base, 0);
      if (base >= n_rays) exhausted = true;
      uint32_t r = kNone;
      bool to_shade = false;
      if (leader && rid == kNone) {
        const uint32_t k = base + (uint32_t)__popc(idle & lt_mask);
        if (k < n_rays) {
          r = rq ? rq[k] : k;
          const DJob& J = jobs[find_job(jobs, n_jobs, r)];
          if (!rq) start_saved_ray<NB>(J, st, r);
          // a shoebox needs no walk: its hit is found when the ray is shaded
          if (J.geom == OMG_GEOM_BOX) to_shade = true;
        }
      }
      const unsigned bm = __ballot_sync(FULL, to_shade);
      if (to_shade) shade_q[(sh_head + sh_cnt + (uint32_t)__popc(bm & lt_mask)) % kQ] = r;
      sh_cnt += (uint32_t)__popc(bm);
      __syncwarp();   // the leaders' saved state before the group reads it
      uint32_t wr = __shfl_sync(FULL, to_shade ? kNone : r, gbase);
      if (wr != kNone) start_walk(wr);
    }
    walking = __ballot_sync(FULL, leader && rid != kNone);
    if (!walking && !sh_cnt && !wk_cnt && (exhausted || parking)) break;

    // ---- cooperative walk steps, until a walk ends or walk_budget steps (none
    // when no group of the warp walks: rays may only be waiting to be shaded)
    for (int step = 0; step < walk_budget; step++) {
      if (__ballot_sync(FULL, rid != kNone) == 0u) break;
      const bool wk = rid != kNone;   // the same in the 4 lanes of a group
      bool out_of_budget = false;
      if (wk) {
        if (budget == 0u) out_of_budget = true;
        else budget--;
      }
      float tk = FLT_MAX;
      int ref = kEmpty4;
      bool hit = false;
      if (wk && !out_of_budget && cur != kDoneC) {
        const float4* c = nodes + 8 * cur + 2 * sub;
        const float4 a = __ldg(c), b = __ldg(c + 1);
        ref = __float_as_int(b.z);
        hit = ref != kEmpty4 && ray_aabb(a.x, a.y, a.z, a.w, b.x, b.y, ox, oy, oz, ix, iy, iz, t_cull, tk);
      }
      // leaves: each lane tests its hit leaf from the group's best, then the
      // group keeps the best of its lanes under the near-tie rule
      const bool leaf = hit && ref < 0;
      if (__ballot_sync(FULL, leaf)) {
        bool lh = have;
        float lt = t_best, lc = t_cull;
        uint32_t ls = s_best, ltr = tri_best;
        int lp = prim_best;
        TieState lts = ts;
        if (leaf) leaf_test<true>(prims, ref, ox, oy, oz, dx, dy, dz, lh, lt, lc, lp, ls, ltr, lts, pwt);
#pragma unroll
        for (int m = 1; m <= 2; m <<= 1) {
          const bool oh = __shfl_xor_sync(FULL, (int)lh, m) != 0;
          const float ot = __shfl_xor_sync(FULL, lt, m);
          const uint32_t os = __shfl_xor_sync(FULL, ls, m);
          const uint32_t otr = __shfl_xor_sync(FULL, ltr, m);
          const int op = __shfl_xor_sync(FULL, lp, m);
          const float omin = __shfl_xor_sync(FULL, lts.t_min, m);
          const bool oamb = __shfl_xor_sync(FULL, (int)lts.amb, m) != 0;
          tie_merge(lh, lt, ls, ltr, lp, lts.t_min, lts.amb, oh, ot, os, otr, op, omin, oamb, ts.fixed);
        }
        if (wk) {
          have = lh;
          t_best = lt;
          s_best = ls;
          tri_best = ltr;
          prim_best = lp;
          ts.t_min = lts.t_min;
          ts.amb = lts.amb;
          if (!ts.fixed) t_cull = lh ? ts.t_min * (1.0f + kTieRel) : FLT_MAX;
        }
      }
      // internal children still in reach, ranked by (entry distance, child)
      const bool in = hit && ref >= 0 && !(tk > t_cull);
      const unsigned vm = __ballot_sync(FULL, in) & (0xFu << gbase);
      const int nv = __popc(vm);
      int rank = 0;
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const float tj = __shfl_sync(FULL, tk, gbase + j);
        if (((vm >> (gbase + j)) & 1u) && (tj < tk || (tj == tk && (uint32_t)j < sub))) rank++;
      }
      const unsigned near_m = __ballot_sync(FULL, in && rank == 0) & (0xFu << gbase);
      const int nxt = __shfl_sync(FULL, ref, near_m ? __ffs(near_m) - 1 : lane);
      if (wk && !out_of_budget && cur != kDoneC && nv > 1) {
        // the others, farthest at the bottom
        if (sp + nv - 1 <= STACK_DEPTH) {
          if (in && rank > 0) {
            sref[sp + nv - 1 - rank] = ref;
            sst[sp + nv - 1 - rank] = tk;
          }
          sp += nv - 1;
        } else if (leader) {
          atomicOr(err, 1u);
        }
      }
      __syncwarp();
      if (wk) {
        if (out_of_budget) {
          if (leader) atomicOr(err, 4u);
          cur = kDoneC;
        } else if (near_m) {
          cur = nxt;
        } else {
          cur = kDoneC;
          while (sp > 0) {
            sp--;
            if (sst[sp] > t_cull) continue;
            cur = sref[sp];
            break;
          }
          if (cur == kDoneC && ts.amb && !ts.fixed) {
            // an ambiguous near-tie window: walk again with the final one
            ts.fixed = true;
            t_cull = ts.t_min * (1.0f + kTieRel);
            have = false;
            t_best = FLT_MAX;
            prim_best = -1;
            sp = 0;
            budget = budget0;
            cur = root;
          }
        }
      }
      // finished walks: hit to the ray's record, id to the shading queue
      const bool fin = wk && cur == kDoneC;
      const unsigned fm = __ballot_sync(FULL, fin && leader);
      if (fin && leader) {
        st.hit[rid] = make_float2(t_best, __int_as_float(have ? prim_best : -1));
        shade_q[(sh_head + sh_cnt + (uint32_t)__popc(fm & lt_mask)) % kQ] = rid;
      }
      if (fin) rid = kNone;
      sh_cnt += (uint32_t)__popc(fm);
      __syncwarp();
      if (fm) break;   // refill the group (and shade once 32 wait)
    }
  }
}

}  // namespace

// A warp owns at most 8 walking rays + 31 waiting for shading when it fetches
// (only with an empty walk queue), so at most 39 rays at any time: each
// queue of 64 ids suffices.
cudaError_t launch_trace_coop(const DJob* jobs, uint32_t n_jobs, uint32_t total_rays, uint32_t max_nb,
                              const DScene* scenes, const DMat* job_mats, const DPanel* panels,
                              const DPanelGroup* groups, float* acc, DLaunch* hdr, uint32_t* job_segments,
                              const LaunchShape& shape, int n_sms, const EpochArgs& ea, cudaStream_t s) {
  if (n_jobs == 0 || total_rays == 0) return cudaSuccess;
  constexpr uint32_t kThreads = 256;
  uint64_t want = (uint64_t)n_sms * (shape.blocks_per_sm ? shape.blocks_per_sm : 4u);
  uint64_t need = ((uint64_t)total_rays + 63u) / 64u;   // 8 warps x 8 walking rays
  uint32_t blocks = (uint32_t)(want < need ? want : need);
  if (blocks == 0) blocks = 1;
  const int steps = shape.walk_steps == 0 ? 1000000 : (int)shape.walk_steps;
  const uint32_t shade_min = shape.wl_shade_min == 0 ? 32u : (shape.wl_shade_min > 32 ? 32u : shape.wl_shade_min);
  if (max_nb <= 3)
    trace_coop_kernel<3><<<blocks, kThreads, 0, s>>>(jobs, n_jobs, total_rays, scenes, job_mats, panels, groups,
                                                     acc, hdr, job_segments, steps, shade_min, ea);
  else
    trace_coop_kernel<8><<<blocks, kThreads, 0, s>>>(jobs, n_jobs, total_rays, scenes, job_mats, panels, groups,
                                                     acc, hdr, job_segments, steps, shade_min, ea);
  return cudaGetLastError();
}

}  // namespace omg
