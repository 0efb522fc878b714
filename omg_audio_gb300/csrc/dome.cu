// Ambient-dome fan on the GPU (crates/omg-scene/src/dome.rs:293-478).
//
// One thread per (listener, fan ray) traces the specular escape
// (trace_escape, dome.rs:330-382: <= max_events mesh hits or pane crossings,
// 80 m horizon); one warp per ray then adds, when the escape is not
// near-full, the straight-through mass-law seep (trace_through,
// dome.rs:390-422, over segment_hits, mesh.rs:546-604). A third kernel bins
// the rays of each listener in fan order (dome.rs:452-458,
// the same f32 sums in the same order), applies the per-listener EMA and
// writes the 9 bins. The fan is deterministic, so the result is too.
#include "device_common.cuh"
#include "walk.cuh"

namespace omg {

namespace {

constexpr float PI_F = 3.14159265358979323846f;
constexpr uint32_t kMaxCross = 64;   // crossings kept per straight-through segment

// dome.rs:56-68
__device__ __forceinline__ bool panel_hit(const DDomePanel& p, float ox, float oy, float oz, float dx, float dy,
                                          float dz, float t_max, float& tout) {
  const float po = p.axis == 0 ? ox : oy, pd = p.axis == 0 ? dx : dy;
  if (fabsf(pd) < 1e-8f) return false;
  const float t = (p.plane - po) / pd;
  if (t < 1e-4f || t >= t_max) return false;
  const float lat = p.axis == 0 ? oy + t * dy : ox + t * dx;
  const float z = oz + t * dz;
  if (lat > p.lat0 && lat < p.lat1 && z > p.z0 && z < p.z1) {
    tout = t;
    return true;
  }
  return false;
}

// The escape of one fan ray as a state machine around its closest-hit walks
// (trace_escape, one event at a time): the ray's position, direction and
// throughput, and how many events it has taken.
struct EscapeRay {
  float px, py, pz, dx, dy, dz;
  float tp[MAXB];
  uint32_t ev;
};

// One event of trace_escape (dome.rs:336-381) after its closest-hit walk:
// mesh hit (mh, tm, prim) or none. Returns 0 when the ray goes on (the next
// walk starts from its new position), 1 when it escaped, 2 when it ends
// without escaping. The same f32 operations as trace_escape.
__device__ __forceinline__ int escape_event(const DScene& S, const DDomeLaunch& L, EscapeRay& r, bool mh, float tm,
                                            int prim) {
  const uint32_t nb = L.nb;
  const float t_mesh = mh ? tm : FLT_MAX;
  float t_pan = t_mesh;
  int pan = -1;
  for (uint32_t k = 0; k < L.n_panels; k++) {
    float t;
    if (panel_hit(L.panels[k], r.px, r.py, r.pz, r.dx, r.dy, r.dz, t_pan, t)) {
      t_pan = t;
      pan = (int)k;
    }
  }
  if (pan >= 0) {
    const DDomePanel& P = L.panels[pan];
    if (!P.glass) return 2;  // a door leaf blocks
#pragma unroll
    for (int b = 0; b < MAXB; b++)
      if ((uint32_t)b < nb) r.tp[b] = r.tp[b] * P.t2[b];
    const float adv = t_pan + 1e-3f;
    r.px = r.px + r.dx * adv;
    r.py = r.py + r.dy * adv;
    r.pz = r.pz + r.dz * adv;
    return 0;
  }
  const bool escaped = r.pz > -0.05f || r.dz > 0.05f;
  if (!mh) return escaped ? 1 : 2;
  if (tm > 80.0f) return escaped ? 1 : 2;
  const float4 p0 = __ldg(S.prims + 3 * prim);
  const float4 p1 = __ldg(S.prims + 3 * prim + 1);
  const DMat& M = S.mats[__float_as_uint(p0.w)];
#pragma unroll
  for (int b = 0; b < MAXB; b++)
    if ((uint32_t)b < nb) r.tp[b] = r.tp[b] * (1.0f - M.absorption[b]);
  if (r.tp[1] < 2e-3f) return 2;
  const float4 nn = __ldg(S.normals + __float_as_uint(p1.w));
  const float nx = nn.x, ny = nn.y, nz = nn.z;
  const float dn = r.dx * nx + r.dy * ny + r.dz * nz;
  float ox = nx, oy = ny, oz = nz;
  if (dn > 0.0f) { ox = nx * -1.0f; oy = ny * -1.0f; oz = nz * -1.0f; }
  const float hx = r.px + r.dx * tm, hy = r.py + r.dy * tm, hz = r.pz + r.dz * tm;
  const float k2 = 2.0f * dn;
  r.dx = r.dx - nx * k2;
  r.dy = r.dy - ny * k2;
  r.dz = r.dz - nz * k2;
  normalize3(r.dx, r.dy, r.dz);
  r.px = hx + ox * 1e-3f;
  r.py = hy + oy * 1e-3f;
  r.pz = hz + oz * 1e-3f;
  return 0;
}

// dome.rs:328-382 under the reference's first-found rule (tie_mode 0): each
// event's closest hit by the reference's ordered walk. Returns true (escaped)
// with the throughput in tp.
__device__ bool trace_escape(const DScene& S, const DDomeLaunch& L, float px, float py, float pz, float dx, float dy,
                             float dz, float tp[MAXB], uint32_t& events) {
  EscapeRay r{px, py, pz, dx, dy, dz, {}, 0u};
#pragma unroll
  for (int b = 0; b < MAXB; b++) r.tp[b] = 1.0f;
  int e = 2;
  for (uint32_t ev = 0; ev < L.max_events; ev++) {
    events++;
    float tm = FLT_MAX;
    int prim = 0;
    const bool mh = mesh_closest<false>(S, r.px, r.py, r.pz, r.dx, r.dy, r.dz, tm, prim, &L.hdr->error);
    e = escape_event(S, L, r, mh, tm, prim);
    if (e != 0) break;
  }
#pragma unroll
  for (int b = 0; b < MAXB; b++) tp[b] = r.tp[b];
  return e == 1;
}

// The specular escape of every (listener, fan ray) under the near-tie rule,
// one lane each, with the persistent tracer's walk: the node phase lane by
// lane (walk_spec_nodes, the grown binary boxes), then the pending leaves
// tested by the whole warp (coop_leaf_rounds). The closest hit under this
// rule does not depend on the walk, so each event sees the hit
// any other near-tie walk finds; the events follow in trace_escape's f32 operations. Lanes
// past the last ray take part in the warp's leaf rounds only.
constexpr uint32_t kEscThreads = 128;
template <bool WT>
__global__ void __launch_bounds__(kEscThreads) dome_escape_walk_kernel(DDomeLaunch L, uint32_t loop_guard) {
  __shared__ uint8_t s_slots[kEscThreads / 32][256];
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t total = L.n_eyes * L.n_rays;
  const DScene& S = *L.scene;
  uint32_t* err = &L.hdr->error;
  EscapeRay r;
  int walk_stack_ref[STACK_DEPTH];
  float walk_stack_t[STACK_DEPTH];
  Walk w;
  w.stack_ref = walk_stack_ref;
  w.stack_t = walk_stack_t;
  w.cur = kDone;
  w.leaf = 0;
  bool active = gid < total && L.max_events > 0;
  int status = 2;
  uint32_t events = 0;
  if (gid < total) {
    const uint32_t eye = gid / L.n_rays, j = gid % L.n_rays;
    const uint32_t i = (uint32_t)((uint64_t)j * L.n_fan / L.n_rays);  // dome.rs:434
    const float4 f = L.fan[i];
    r.px = L.eyes[3 * eye]; r.py = L.eyes[3 * eye + 1]; r.pz = L.eyes[3 * eye + 2];
    r.dx = f.x; r.dy = f.y; r.dz = f.z;
#pragma unroll
    for (int b = 0; b < MAXB; b++) r.tp[b] = 1.0f;
    r.ev = 0;
    if (active) {
      walk_begin<true>(w, S, r.px, r.py, r.pz, r.dx, r.dy, r.dz, false);
      events++;
    }
  }
  uint32_t iters = 0;
  while (__any_sync(0xffffffffu, active)) {
    if (++iters > loop_guard) {
      atomicOr(err, 8u);
      active = false;
      break;
    }
    bool over = false;
    if (active) {
      int st = 1 << 30;   // the node phase runs until the warp's lanes hold leaves (bounded by the walk budget)
      over = walk_spec_nodes(w, S, r.px, r.py, r.pz, r.dx, r.dy, r.dz, st, err);
    }
    coop_leaf_rounds<WT>(w, active && !over, WT ? S.prims_wt : S.prims, WT, r.px, r.py, r.pz, r.dx, r.dy, r.dz,
                         s_slots[threadIdx.x >> 5], kCoopRounds, err);
    if (active) {
      if (!over && w.cur == kDone && w.leaf == 0) over = !walk_restart_fixed(w, S.root, S.walk_budget);
      if (over) {
        const int e = escape_event(S, L, r, walk_have(w), w.t_best, w.prim_best);
        r.ev++;
        if (e != 0) {
          status = e;
          active = false;
        } else if (r.ev >= L.max_events) {
          status = 2;
          active = false;
        } else {
          walk_begin<true>(w, S, r.px, r.py, r.pz, r.dx, r.dy, r.dz, false);
          events++;
        }
      }
    }
  }
  if (gid < total) {
    float* o = L.ray_tp + (uint64_t)gid * L.nb;
    for (uint32_t b = 0; b < L.nb; b++) o[b] = r.tp[b];
    L.ray_escape[gid] = status == 1 ? 1 : 0;
    atomicAdd(&L.events[0], events);
  }
}

// One warp's shared memory for the straight-through segment of one fan ray.
constexpr uint32_t kThroughWarps = 4;        // rays (warps) per block
constexpr uint32_t kWarpStack = 512;         // pending node refs of one warp's walk
constexpr uint32_t kMaxThroughRounds = 1u << 20;
struct ThroughSmem {
  int ref[kWarpStack];
  unsigned long long key[kWarpStack];        // the ref's depth-first position (below)
  float t[kMaxCross];                        // crossings as found
  uint32_t prim[kMaxCross];
  unsigned long long ckey[kMaxCross];
  float st[kMaxCross];                       // crossings sorted
  uint32_t sprim[kMaxCross];
  uint32_t n;
};

// Straight-through seep of one fan ray (trace_through, dome.rs:390-422) by a
// whole warp. The crossings of the 50 m segment (segment_hits,
// mesh.rs:546-604) are collected by a walk in which every lane takes one
// pending ref per round (children whose box the segment meets are pushed
// warp-aggregated, leaves test their primitives), so the any-hit walk, which
// visits every node the segment meets, runs 32 nodes wide instead of one.
//
// The reference sorts the crossings by t with a stable sort over its
// depth-first visiting order (child b before child a) and then merges
// clusters within 1e-4 / max(len, 1) keeping the lowest surface id (the
// first one on equal ids). Each ref therefore carries its depth-first
// position: bit 63 - d set for the a child at depth d (d < 58) above a
// 6-bit depth, so that ordering crossings by (t, key, primitive) reproduces
// the reference's order, and the merge and the transmission product then run
// in that order, uniformly across the warp.
__device__ void through_warp(const DScene& S, const DDomeLaunch& L, ThroughSmem& W, uint32_t lane, float ex,
                             float ey, float ez, float dx, float dy, float dz, float tp[MAXB]) {
  constexpr unsigned FULL = 0xffffffffu;
  const uint32_t nb = L.nb;
  const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
  for (int b = 0; b < MAXB; b++) tp[b] = 1.0f;
  const float bx = ex + dx * 50.0f, by = ey + dy * 50.0f, bz = ez + dz * 50.0f;
  if (bz < -0.05f) {
#pragma unroll
    for (int b = 0; b < MAXB; b++) tp[b] = 0.0f;
    return;
  }
  uint32_t n = 0;
  uint32_t fail = 0;   // error bits: 1 walk overflow, 2 too many crossings
  float len = 0.0f;
  if (S.n_prims != 0) {
    float sx = bx - ex, sy = by - ey, sz = bz - ez;
    len = sqrtf(sx * sx + sy * sy + sz * sz);
    if (len >= 1e-6f) {
      const float il = __frcp_rn(len);
      sx = sx * il;
      sy = sy * il;
      sz = sz * il;
      const float ix = __frcp_rn(sx), iy = __frcp_rn(sy), iz = __frcp_rn(sz);
      if (lane == 0) {
        W.ref[0] = S.root;
        W.key[0] = 0ull;
        W.n = 0u;
      }
      __syncwarp();
      uint32_t sp = 1, rounds = 0;
      while (sp > 0) {
        if (++rounds > kMaxThroughRounds) {
          fail |= 1u;
          break;
        }
        const uint32_t take = sp < 32u ? sp : 32u;
        const uint32_t base = sp - take;
        const bool act = lane < take;
        int cur = 0;
        unsigned long long key = 0ull;
        if (act) {
          cur = W.ref[base + lane];
          key = W.key[base + lane];
        }
        __syncwarp();
        sp = base;
        bool h0 = false, h1 = false;
        int c0 = 0, c1 = 0;
        if (act && cur >= 0) {
          const float4 n0 = __ldg(S.nodes + 4 * cur + 0);
          const float4 n1 = __ldg(S.nodes + 4 * cur + 1);
          const float4 n2 = __ldg(S.nodes + 4 * cur + 2);
          const float4 n3 = __ldg(S.nodes + 4 * cur + 3);
          float ta, tb;
          h0 = ray_aabb(n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, ex, ey, ez, ix, iy, iz, len, ta);
          h1 = ray_aabb(n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, ex, ey, ez, ix, iy, iz, len, tb);
          c0 = __float_as_int(n3.x);
          c1 = __float_as_int(n3.y);
        }
        const unsigned m0 = __ballot_sync(FULL, h0), m1 = __ballot_sync(FULL, h1);
        const uint32_t tot = (uint32_t)(__popc(m0) + __popc(m1));
        if (sp + tot > kWarpStack) {
          fail |= 1u;
          break;
        }
        const uint32_t d = (uint32_t)(key & 63ull);
        const unsigned long long child = (key & ~63ull) | (unsigned long long)(d < 63u ? d + 1u : 63u);
        const unsigned long long abit = d < 58u ? (1ull << (63u - d)) : 0ull;
        const uint32_t pos = sp + (uint32_t)(__popc(m0 & lt) + __popc(m1 & lt));
        if (h0) {
          W.ref[pos] = c0;
          W.key[pos] = child | abit;
        }
        if (h1) {
          W.ref[pos + (h0 ? 1u : 0u)] = c1;
          W.key[pos + (h0 ? 1u : 0u)] = child;
        }
        sp += tot;
        if (act && cur < 0) {
          const uint32_t code = ~(uint32_t)cur;
          const uint32_t start = code >> 3, end = start + (code & 7u) + 1u;
          for (uint32_t i = start; i < end; i++) {
            const float4 p0 = __ldg(S.prims + 3 * i + 0);
            const float4 p1 = __ldg(S.prims + 3 * i + 1);
            const float4 p2 = __ldg(S.prims + 3 * i + 2);
            float t;
            if (ray_tri(p0, p1, p2, ex, ey, ez, sx, sy, sz, t)) {
              const float tt = t / len;
              if (tt > 1e-4f && tt < 1.0f - 1e-4f) {
                const uint32_t k = atomicAdd(&W.n, 1u);
                if (k < kMaxCross) {
                  W.t[k] = tt;
                  W.prim[k] = i;
                  W.ckey[k] = key;
                }
              }
            }
          }
        }
        __syncwarp();
      }
      __syncwarp();
      n = W.n;
      if (n > kMaxCross) fail |= 2u;
    }
  }
  if (fail) {
    if (lane == 0) atomicOr(&L.hdr->error, fail);
#pragma unroll
    for (int b = 0; b < MAXB; b++) tp[b] = 0.0f;
    return;
  }
  // rank sort by (t, depth-first key, primitive): every key is distinct
  for (uint32_t e = lane; e < n; e += 32u) {
    const float te = W.t[e];
    const unsigned long long ke = W.ckey[e];
    const uint32_t pe = W.prim[e];
    uint32_t r = 0;
    for (uint32_t q = 0; q < n; q++) {
      const float tq = W.t[q];
      const unsigned long long kq = W.ckey[q];
      if (tq < te || (tq == te && (kq < ke || (kq == ke && W.prim[q] < pe)))) r++;
    }
    W.st[r] = te;
    W.sprim[r] = pe;
  }
  __syncwarp();
  // same-t merge (lowest surface id wins, the cluster keeps its first t),
  // then the mass-law product in crossing order
  const float tol = 1e-4f / fmaxf(len, 1.0f);
  bool open = false;
  float anchor = 0.0f;
  uint32_t wtri = 0, wmat = 0;
  bool dead = false;
  for (uint32_t q = 0; q <= n && !dead; q++) {
    uint32_t tri = 0, mat = 0;
    float tq = 0.0f;
    const bool last = q == n;
    if (!last) {
      const uint32_t pq = W.sprim[q];
      tq = W.st[q];
      mat = __float_as_uint(__ldg(S.prims + 3 * pq + 0).w);
      tri = __float_as_uint(__ldg(S.prims + 3 * pq + 1).w);
      if (open && fabsf(tq - anchor) < tol) {
        if (S.tri_surface[tri] < S.tri_surface[wtri]) {
          wtri = tri;
          wmat = mat;
        }
        continue;
      }
    }
    if (open) {
      const DMat& M = S.mats[wmat];
#pragma unroll
      for (int b = 0; b < MAXB; b++)
        if ((uint32_t)b < nb) tp[b] = tp[b] * M.t2[b];
      if (tp[0] < 1e-7f) dead = true;
    }
    anchor = tq;
    wtri = tri;
    wmat = mat;
    open = true;
  }
  if (dead) {
#pragma unroll
    for (int b = 0; b < MAXB; b++) tp[b] = 0.0f;
    return;
  }
  for (uint32_t k = 0; k < L.n_panels; k++) {
    float t;
    if (panel_hit(L.panels[k], ex, ey, ez, dx, dy, dz, 80.0f, t)) {
#pragma unroll
      for (int b = 0; b < MAXB; b++)
        if ((uint32_t)b < nb) tp[b] = tp[b] * L.panels[k].t2[b];
    }
  }
}

// The specular escape of every (listener, fan ray) under the first-found
// rule, one thread each: its transmission goes to ray_tp and its escape flag
// to ray_escape; the straight-through kernel then completes the rays that
// need it.
__global__ void dome_escape_kernel(DDomeLaunch L) {
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= L.n_eyes * L.n_rays) return;
  const uint32_t eye = gid / L.n_rays, j = gid % L.n_rays;
  const DScene S = *L.scene;
  const uint32_t i = (uint32_t)((uint64_t)j * L.n_fan / L.n_rays);  // dome.rs:434
  const float4 f = L.fan[i];
  const float ex = L.eyes[3 * eye], ey = L.eyes[3 * eye + 1], ez = L.eyes[3 * eye + 2];
  float bp[MAXB];
  uint32_t events = 0;
  const bool esc = trace_escape(S, L, ex, ey, ez, f.x, f.y, f.z, bp, events);
  float* o = L.ray_tp + (uint64_t)gid * L.nb;
  for (uint32_t b = 0; b < L.nb; b++) o[b] = bp[b];
  L.ray_escape[gid] = esc ? 1 : 0;
  atomicAdd(&L.events[0], events);
}

// dome.rs:432-446 per ray: a near-full escape stands; otherwise the
// straight-through seep, combined with an escape by the per-band max. One
// warp per ray.
__global__ void __launch_bounds__(32 * kThroughWarps) dome_through_kernel(DDomeLaunch L) {
  __shared__ ThroughSmem smem[kThroughWarps];
  const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
  const uint64_t gid = (uint64_t)blockIdx.x * kThroughWarps + wib;
  if (gid >= (uint64_t)L.n_eyes * L.n_rays) return;   // warp-uniform
  const uint32_t nb = L.nb;
  float* o = L.ray_tp + gid * nb;
  const bool esc = L.ray_escape[gid] != 0;
  float bp[MAXB];
#pragma unroll
  for (int b = 0; b < MAXB; b++) bp[b] = (uint32_t)b < nb ? o[b] : 0.0f;
  if (esc && bp[0] > 0.5f) return;
  const uint32_t eye = (uint32_t)(gid / L.n_rays), j = (uint32_t)(gid % L.n_rays);
  const uint32_t i = (uint32_t)((uint64_t)j * L.n_fan / L.n_rays);
  const float4 f = L.fan[i];
  const float ex = L.eyes[3 * eye], ey = L.eyes[3 * eye + 1], ez = L.eyes[3 * eye + 2];
  float tp[MAXB];
  through_warp(*L.scene, L, smem[wib], lane, ex, ey, ez, f.x, f.y, f.z, tp);
  if (esc) {
#pragma unroll
    for (int b = 0; b < MAXB; b++) tp[b] = fmaxf(tp[b], bp[b]);
  }
  __syncwarp();
  if (lane == 0) {
    for (uint32_t b = 0; b < nb; b++) o[b] = tp[b];
    atomicAdd(&L.events[1], 1u);
  }
}

// dome.rs:452-477 per listener: bins in fan order, EMA, directions. The
// block stages the listener's rays kDomeChunk at a time: every thread turns
// one ray into its terms (tp / n_rays per band, the direction weighted by
// max(tp[1], 0.2 tp[0]), its bin, or no bin when tp[0] <= 1e-9); then lane
// k < 9 of the first warp adds the terms of bin k's rays in fan order (the
// same f32 sums in the same order as the reference's one loop), finding them
// 32 at a time by ballots.
constexpr uint32_t kDomeChunk = 256;
constexpr uint32_t kDomeBinThreads = 128;
__global__ void __launch_bounds__(kDomeBinThreads) dome_bins_kernel(DDomeLaunch L, float ema_alpha) {
  __shared__ float s_c[kDomeChunk * MAXB];
  __shared__ float s_w[kDomeChunk * 3];
  __shared__ uint32_t s_bin[kDomeChunk];
  const uint32_t eye = blockIdx.x;
  const uint32_t k = threadIdx.x;  // bin 0..8 in the first warp
  const uint32_t nb = L.nb;
  const bool primed = L.primed[eye] != 0u;
  float e[MAXB];
#pragma unroll
  for (int b = 0; b < MAXB; b++) e[b] = 0.0f;
  float sx = 0.0f, sy = 0.0f, sz = 0.0f;
  const float nr = (float)L.n_rays;
  const float* tp_eye = L.ray_tp + (uint64_t)eye * L.n_rays * nb;
  for (uint32_t j0 = 0; j0 < L.n_rays; j0 += kDomeChunk) {
    const uint32_t m = L.n_rays - j0 < kDomeChunk ? L.n_rays - j0 : kDomeChunk;
    for (uint32_t q = threadIdx.x; q < m; q += blockDim.x) {
      const float4 f = L.fan[(uint32_t)((uint64_t)(j0 + q) * L.n_fan / L.n_rays)];
      const float* tp = tp_eye + (uint64_t)(j0 + q) * nb;
      const float t0 = tp[0];
      if (t0 > 1e-9f) {
        for (uint32_t b = 0; b < nb; b++) s_c[q * nb + b] = tp[b] / nr;
        const float w = fmaxf(tp[1], t0 * 0.2f);
        s_w[3 * q] = f.x * w;
        s_w[3 * q + 1] = f.y * w;
        s_w[3 * q + 2] = f.z * w;
        s_bin[q] = (uint32_t)__float_as_int(f.w);
      } else {
        s_bin[q] = 0xFFFFFFFFu;
      }
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      for (uint32_t q0 = 0; q0 < m; q0 += 32) {
        const uint32_t my_bin = q0 + k < m ? s_bin[q0 + k] : 0xFFFFFFFFu;
        uint32_t mine = 0;
        for (uint32_t bin = 0; bin < 9; bin++) {
          const uint32_t bm = __ballot_sync(0xffffffffu, my_bin == bin);
          if (k == bin) mine = bm;
        }
        while (mine) {
          const uint32_t q = q0 + (uint32_t)(__ffs(mine) - 1);
          mine &= mine - 1u;
#pragma unroll
          for (int b = 0; b < MAXB; b++)
            if ((uint32_t)b < nb) e[b] = e[b] + s_c[q * nb + b];
          sx = sx + s_w[3 * q];
          sy = sy + s_w[3 * q + 1];
          sz = sz + s_w[3 * q + 2];
        }
      }
    }
    __syncthreads();
  }
  if (k < 9) {
    const float alpha = primed ? ema_alpha : 1.0f;
    float* ema = L.ema + ((uint64_t)eye * 9 + k) * nb;
    for (uint32_t b = 0; b < nb; b++) {
      L.raw[((uint64_t)eye * 9 + k) * nb + b] = e[b];
      ema[b] = ema[b] + alpha * (e[b] - ema[b]);
      L.out_energy[((uint64_t)eye * 9 + k) * nb + b] = ema[b];
    }
    float dxo, dyo, dzo;
    if (sqrtf(sx * sx + sy * sy + sz * sz) > 1e-6f) {
      dxo = sx; dyo = sy; dzo = sz;
      normalize3(dxo, dyo, dzo);
    } else if (k == 8) {
      dxo = 0.0f; dyo = 0.0f; dzo = 1.0f;
    } else {
      const float az = ((float)k + 0.5f) * TAU_F / 8.0f - PI_F;
      double sn, cs;
      sincos((double)az, &sn, &cs);
      dxo = (float)cs; dyo = (float)sn; dzo = 0.0f;
    }
    float* od = L.out_dir + ((uint64_t)eye * 9 + k) * 3;
    od[0] = dxo;
    od[1] = dyo;
    od[2] = dzo;
  }
  __syncthreads();
  if (k == 0) L.primed[eye] = 1u;
}

// dome.rs:316-324 fan + dome.rs:304-310 bin per direction (in .w)
__global__ void fan_kernel(float4* fan, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float ga = PI_F * (3.0f - sqrtf(5.0f));
  const float z = 1.0f - 2.0f * ((float)i + 0.5f) / (float)n;
  const float r = sqrtf(fmaxf(1.0f - z * z, 0.0f));
  const float phi = ga * (float)i;
  double s, c;
  sincos((double)phi, &s, &c);
  const float x = r * (float)c, y = r * (float)s;
  int bin;
  if (z > 0.87f) {
    bin = 8;
  } else {
    const float az = (float)atan2((double)y, (double)x) + PI_F;
    const float q = az / (TAU_F / 8.0f);
    uint32_t b = q >= 0.0f ? (uint32_t)q : 0u;
    bin = (int)(b < 7u ? b : 7u);
  }
  fan[i] = make_float4(x, y, z, __int_as_float(bin));
}

}  // namespace

cudaError_t build_dome_fan(float4* fan, uint32_t n, cudaStream_t s) {
  fan_kernel<<<(n + 127) / 128, 128, 0, s>>>(fan, n);
  return cudaGetLastError();
}

cudaError_t launch_dome(const DDomeLaunch& L, cudaStream_t s) {
  const uint64_t total = (uint64_t)L.n_eyes * L.n_rays;
  if (total == 0) return cudaSuccess;
  if (L.tie && L.wt)
    dome_escape_walk_kernel<true><<<(uint32_t)((total + kEscThreads - 1) / kEscThreads), kEscThreads, 0, s>>>(
        L, kDefaultLoopGuard);
  else if (L.tie)
    dome_escape_walk_kernel<false><<<(uint32_t)((total + kEscThreads - 1) / kEscThreads), kEscThreads, 0, s>>>(
        L, kDefaultLoopGuard);
  else
    dome_escape_kernel<<<(uint32_t)((total + 127) / 128), 128, 0, s>>>(L);
  dome_through_kernel<<<(uint32_t)((total + kThroughWarps - 1) / kThroughWarps), 32 * kThroughWarps, 0, s>>>(L);
  dome_bins_kernel<<<L.n_eyes, kDomeBinThreads, 0, s>>>(L, 0.35f);
  return cudaGetLastError();
}

}  // namespace omg
