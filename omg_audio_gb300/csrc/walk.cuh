// The per-lane closest-hit walk of the persistent tracer (trace.cu) and of the
// dome's escape walk (dome.cu): a walk that stops after a step budget and
// resumes, the near-tie rule on a compact state, the speculative node phase
// on the grown boxes, and the pending leaves tested by the whole warp.
#pragma once
#include "device_common.cuh"

namespace omg {

namespace {

// Per-lane closest-hit walk that can stop after a step budget and resume
// (mesh.rs:484-541 semantics; TIE as in mesh_closest).
// The walk's scalars stay in registers (the struct has no arrays, so it is
// split into registers once inlined); the two stacks live beside it.
struct Walk {
  int cur;
  int leaf;          // postponed leaf (TIE), or 0
  int sp;
  int prim_best;     // the winner so far (-1: no hit yet)
  float t_best;
  float t_min;       // TIE: exact nearest hit so far (FLT_MAX: none); the window is t_min (1 + 1e-6)
  uint32_t flags;    // TIE: kWalkAmb, kWalkFixed (TieState, device_common.cuh); kWalkFast
  float ix, iy, iz;
  uint32_t budget;
  int* stack_ref;
  float* stack_t;
};
// The near-tie state is kept compact (the winner's surface and triangle ids
// are read back from its primitive when a comparison needs them, the culling
// bound is recomputed from t_min): the walk's scalars live in registers next
// to the ray's, under the persistent kernels' 64-register cap.
constexpr uint32_t kWalkAmb = 1u, kWalkFixed = 2u;
// the fused multiply-add slab test applies (origin within the margin, no d_a near 0)
constexpr uint32_t kWalkFast = 4u;

__device__ __forceinline__ bool walk_have(const Walk& w) { return w.prim_best >= 0; }

// Culling bound. TIE: the near-tie window (infinite before the first hit);
// otherwise the best t (the reference's strict culling).
template <bool TIE>
__device__ __forceinline__ float walk_cull(const Walk& w) {
  return TIE ? w.t_min * (1.0f + kTieRel) : (w.prim_best >= 0 ? w.t_best : FLT_MAX);
}

constexpr int kDone = 0x7FFFFFFF;  // never a node index (< 2^28)
constexpr int kMaxWarps = 8;       // warps of a trace_kernel block (at most 256 threads)
constexpr int kCoopRounds = 8;     // cooperative leaf rounds per loop iteration

template <bool TIE>
__device__ __forceinline__ int walk_pop(Walk& w) {
  const float cull = walk_cull<TIE>(w);
  while (w.sp > 0) {
    w.sp--;
    if (TIE ? w.stack_t[w.sp] > cull : (walk_have(w) && w.stack_t[w.sp] >= w.t_best)) continue;
    return w.stack_ref[w.sp];
  }
  return kDone;
}

template <bool TIE>
__device__ __forceinline__ void walk_begin(Walk& w, const DScene& S, float ox, float oy, float oz, float dx, float dy,
                                           float dz, bool wide) {
  // the 4-wide tree (when asked for, and the scene has one) where the
  // near-tie rule lets the visit order differ
  w.cur = S.n_prims ? ((TIE && wide && S.nodes4) ? S.root4 : S.root) : kDone;
  w.leaf = 0;
  w.sp = 0;
  w.prim_best = -1;
  w.t_best = FLT_MAX;
  w.t_min = FLT_MAX;
  w.ix = __frcp_rn(dx);
  w.iy = __frcp_rn(dy);
  w.iz = __frcp_rn(dz);
  // the margin 2^-19 M_a covers the fma slab test's rounding for |o_a| <= 7 M_a;
  // the test also needs finite products (no direction component near 0)
  const float kTiny = 8.673617379884035e-19f;   // 2^-60
  const bool fast = fabsf(ox) <= 7.0f * S.fast_m[0] && fabsf(oy) <= 7.0f * S.fast_m[1] &&
                    fabsf(oz) <= 7.0f * S.fast_m[2] && fabsf(dx) >= kTiny && fabsf(dy) >= kTiny && fabsf(dz) >= kTiny;
  w.flags = fast ? kWalkFast : 0u;
  w.budget = S.walk_budget;
}

// A near-tie walk that ended with an ambiguous window starts over in fixed
// mode from `root` (t_min stays: the window is final); the caller keeps walking.
__device__ __forceinline__ bool walk_restart_fixed(Walk& w, int root, uint32_t budget) {
  if (!(w.flags & kWalkAmb) || (w.flags & kWalkFixed)) return false;
  w.flags |= kWalkFixed;
  w.prim_best = -1;
  w.t_best = FLT_MAX;
  w.cur = root;
  w.leaf = 0;
  w.sp = 0;
  w.budget = budget;
  return true;
}

// One hit of a near-tie walk, primitive i at t with authored surface s and
// original triangle tr (the rule of tie_take, device_common.cuh, on the
// compact state).
__device__ __forceinline__ void walk_take_tie(Walk& w, const float4* __restrict__ prims, uint32_t i, float t,
                                              uint32_t s, uint32_t tr) {
  {
    const bool have = w.prim_best >= 0;
    // the winner's key, read back from its primitive
    auto less_than_best = [&]() {
      const uint32_t bs = __float_as_uint(__ldg(prims + 3 * w.prim_best + 2).w);
      const uint32_t btr = __float_as_uint(__ldg(prims + 3 * w.prim_best + 1).w);
      return tie_key_less(s, tr, t, bs, btr, w.t_best);
    };
    bool take;
    if (w.flags & kWalkFixed) {
      take = t <= w.t_min * (1.0f + kTieRel) && (!have || less_than_best());
    } else if (!have) {
      take = true;
      w.t_min = t;
    } else if (t < w.t_min) {
      const float win = t * (1.0f + kTieRel);
      if (w.t_best <= win) {
        take = less_than_best();
      } else {
        if (w.t_min <= win) w.flags |= kWalkAmb;
        take = true;
      }
      w.t_min = t;
    } else {
      take = t <= w.t_min * (1.0f + kTieRel) && less_than_best();
    }
    if (take) {
      w.prim_best = (int)i;
      w.t_best = t;
    }
  }
}

// One leaf of a near-tie walk, its primitives in order (prims: the exact
// vertices in watertight contexts, wt).
__device__ __forceinline__ void walk_leaf_tie(Walk& w, const float4* __restrict__ prims, int leaf, float ox,
                                              float oy, float oz, float dx, float dy, float dz, bool wt) {
  const uint32_t code = ~(uint32_t)leaf;
  const uint32_t start = code >> 3, end = start + (code & 7u) + 1u;
  for (uint32_t i = start; i < end; i++) {
    const float4 p0 = __ldg(prims + 3 * i + 0);
    const float4 p1 = __ldg(prims + 3 * i + 1);
    const float4 p2 = __ldg(prims + 3 * i + 2);
    float t;
    if (!tri_hit(wt, p0, p1, p2, ox, oy, oz, dx, dy, dz, t)) continue;
    walk_take_tie(w, prims, i, t, __float_as_uint(p2.w), __float_as_uint(p1.w));
  }
}

// Up to `steps` node steps of the 4-wide walk (mesh_closest4 in pieces).
__device__ __forceinline__ bool walk4_steps(Walk& w, const DScene& S, float ox, float oy, float oz, float dx,
                                            float dy, float dz, int steps, uint32_t* err) {
  while (steps-- > 0) {
    if (w.cur == kDone) {
      if (!walk_restart_fixed(w, S.root4, S.walk_budget)) break;
      continue;
    }
    if (w.budget-- == 0u) {
      atomicOr(err, 4u);
      w.cur = kDone;
      w.flags &= ~kWalkAmb;
      break;
    }
    // the compact state expanded for the generic 4-wide step
    bool have = walk_have(w);
    float t_cull = walk_cull<true>(w);
    int pb = w.prim_best;
    uint32_t sb = 0, tb = 0;
    if (have) {
      sb = __float_as_uint(__ldg(S.prims + 3 * pb + 2).w);
      tb = __float_as_uint(__ldg(S.prims + 3 * pb + 1).w);
    }
    TieState ts;
    ts.t_min = w.t_min;
    ts.amb = (w.flags & kWalkAmb) != 0u;
    ts.fixed = (w.flags & kWalkFixed) != 0u;
    w.cur = bvh4_step(S.nodes4, S.prims_wt ? S.prims_wt : S.prims, w.cur, ox, oy, oz, dx, dy, dz, w.ix, w.iy, w.iz,
                      have, w.t_best, t_cull, pb, sb, tb, ts, w.stack_ref, w.stack_t, w.sp, err,
                      S.prims_wt != nullptr);
    w.prim_best = have ? pb : -1;
    w.t_min = ts.t_min;
    w.flags = (w.flags & kWalkFast) | (ts.amb ? kWalkAmb : 0u) | (ts.fixed ? kWalkFixed : 0u);
  }
  if (w.cur == kDone) walk_restart_fixed(w, S.root4, S.walk_budget);
  return w.cur == kDone;
}

// The node phase of the near-tie walk (TIE = true): speculative while-while
// descent over the grown boxes with the fused multiply-add slab test,
// postponing one leaf, until every lane of the warp holds a leaf (or has none
// left to reach). A ray whose origin lies beyond the boxes' margin (|o_a| >
// 7 M_a: never in a trace that starts inside the scene) or that runs along a
// coordinate plane (a direction component of 0) uses the plain slab test on
// the same grown boxes. Returns true when the walk ran out of its budget (it
// is then over, flag 4 raised).
__device__ __forceinline__ bool walk_spec_nodes(Walk& w, const DScene& S, float ox, float oy, float oz, float dx,
                                                float dy, float dz, int& steps, uint32_t* err) {
  const float4* __restrict__ tnodes = S.nodes_f;
  while (steps > 0 && w.cur >= 0 && w.cur != kDone) {
    steps--;
    if (w.budget-- == 0u) {
      atomicOr(err, 4u);
      w.cur = kDone;
      w.leaf = 0;
      return true;
    }
    const float4 n0 = __ldg(tnodes + 4 * w.cur + 0);
    const float4 n1 = __ldg(tnodes + 4 * w.cur + 1);
    const float4 n2 = __ldg(tnodes + 4 * w.cur + 2);
    const float4 n3 = __ldg(tnodes + 4 * w.cur + 3);
    const float tmax = walk_cull<true>(w);   // infinite before the first hit; the final window in fixed mode
    float ta, tb;
    bool h0, h1;
    if (w.flags & kWalkFast) {
      const float oix = ox * w.ix, oiy = oy * w.iy, oiz = oz * w.iz;
      h0 = ray_aabb_fma(n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, oix, oiy, oiz, w.ix, w.iy, w.iz, tmax, ta);
      h1 = ray_aabb_fma(n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, oix, oiy, oiz, w.ix, w.iy, w.iz, tmax, tb);
    } else {
      h0 = ray_aabb(n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, ox, oy, oz, w.ix, w.iy, w.iz, tmax, ta);
      h1 = ray_aabb(n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, ox, oy, oz, w.ix, w.iy, w.iz, tmax, tb);
    }
    const int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
    if (h0 && h1) {
      int nr, fr;
      float ft;
      if (ta <= tb) { nr = c0; fr = c1; ft = tb; }
      else { nr = c1; fr = c0; ft = ta; }
      if (w.sp < STACK_DEPTH) {
        w.stack_ref[w.sp] = fr;
        w.stack_t[w.sp] = ft;
        w.sp++;
      } else {
        atomicOr(err, 1u);
      }
      w.cur = nr;   // the nearer entry t <= tmax = t_cull: never culled here
    } else if (h0) {
      w.cur = c0;
    } else if (h1) {
      w.cur = c1;
    } else {
      w.cur = walk_pop<true>(w);
    }
    if (w.cur < 0 && w.leaf == 0) {
      w.leaf = w.cur;
      w.cur = walk_pop<true>(w);
    }
    if (__all_sync(__activemask(), w.leaf < 0 || w.cur == kDone)) break;
  }
  if (w.leaf == 0 && w.cur < 0) {
    w.leaf = w.cur;
    w.cur = walk_pop<true>(w);
  }
  return false;
}

// The near-tie walk (TIE = true): speculative while-while over the grown
// boxes with the fused multiply-add slab test (walk_spec_nodes), then the
// postponed leaves one after another.
__device__ __forceinline__ bool walk_spec(Walk& w, const DScene& S, float ox, float oy, float oz, float dx,
                                          float dy, float dz, int steps, uint32_t* err) {
  const bool wt = S.prims_wt != nullptr;
  const float4* __restrict__ prims = wt ? S.prims_wt : S.prims;
  if (walk_spec_nodes(w, S, ox, oy, oz, dx, dy, dz, steps, err)) return true;
  while (w.leaf < 0 && steps > 0) {
    steps--;
    if (w.budget-- == 0u) {
      atomicOr(err, 4u);
      w.cur = kDone;
      w.leaf = 0;
      return true;
    }
    walk_leaf_tie(w, prims, w.leaf, ox, oy, oz, dx, dy, dz, wt);
    w.leaf = 0;
    if (w.cur < 0) {
      w.leaf = w.cur;
      w.cur = walk_pop<true>(w);
    }
  }
  if (w.cur == kDone && w.leaf == 0) {
    // an ambiguous near-tie window: the walk starts over in fixed mode
    return !walk_restart_fixed(w, S.root, S.walk_budget);
  }
  return false;
}

// Leaves of near-tie walks tested by the whole warp (every lane calls this,
// warp-uniformly; `own`: this lane is walking). A leaf holds 1 to 8
// primitives, and one lane testing its own leaf's primitives one after
// another leaves most of the warp idle; here the primitives of every lane's
// pending leaf are laid out in a per-warp slot list (shared memory, `slots`:
// 256 bytes), each lane tests one slot's primitive against the slot owner's
// ray (fetched by shuffles), and each owner then takes its hits in leaf order,
// so the near-tie state sees the sequence walk_leaf_tie would give it. After a
// round, a walk whose next node is a leaf postpones it, and rounds repeat
// while any lane holds a leaf (at most `rounds`).
// WT: the warp may hold walks of watertight scenes (the owner's flag is then
// read); false compiles the reference's test alone.
template <bool WT>
__device__ __forceinline__ void coop_leaf_rounds(Walk& w, bool own_walk, const float4* lane_prims, bool wt,
                                                 float ox, float oy, float oz, float dx, float dy, float dz,
                                                 uint8_t* __restrict__ slots, int rounds, uint32_t* err) {
  const unsigned FULL = 0xffffffffu;
  const uint32_t lane = threadIdx.x & 31u;
  // the owner's primitives, its watertight flag in bit 0 (the arrays are 16-byte aligned)
  const unsigned long long my_prims = reinterpret_cast<unsigned long long>(lane_prims) | ((WT && wt) ? 1ull : 0ull);
  while (rounds-- > 0) {
    bool own = own_walk && w.leaf < 0;
    if (__ballot_sync(FULL, own) == 0u) break;
    uint32_t start = 0, cnt = 0;
    if (own) {
      if (w.budget-- == 0u) {
        // out of budget: the walk is over (and is not walked again)
        atomicOr(err, 4u);
        w.cur = kDone;
        w.leaf = 0;
        w.flags &= ~kWalkAmb;
        own = false;
      } else {
        const uint32_t code = ~(uint32_t)w.leaf;
        start = code >> 3;
        cnt = (code & 7u) + 1u;
        w.leaf = 0;
      }
    }
    // slot ranges: an inclusive scan of the leaf sizes over the warp
    uint32_t inc = cnt;
#pragma unroll
    for (uint32_t d = 1; d < 32u; d <<= 1) {
      const uint32_t v = __shfl_up_sync(FULL, inc, d);
      if (lane >= d) inc += v;
    }
    const uint32_t total = __shfl_sync(FULL, inc, 31);
    const uint32_t excl = inc - cnt;
    const uint32_t kmax = __reduce_max_sync(FULL, cnt);
    for (uint32_t k = 0; k < cnt; k++) slots[excl + k] = (uint8_t)lane;
    __syncwarp();
    for (uint32_t base = 0; base < total; base += 32u) {
      const uint32_t p = base + lane;
      const bool act = p < total;
      const uint32_t o = act ? slots[p] : 0u;
      const uint32_t o_start = __shfl_sync(FULL, start, o), o_excl = __shfl_sync(FULL, excl, o);
      const float rx = __shfl_sync(FULL, ox, o), ry = __shfl_sync(FULL, oy, o), rz = __shfl_sync(FULL, oz, o);
      const float sx = __shfl_sync(FULL, dx, o), sy = __shfl_sync(FULL, dy, o), sz = __shfl_sync(FULL, dz, o);
      const unsigned long long op = __shfl_sync(FULL, my_prims, o);
      const float4* P = reinterpret_cast<const float4*>(WT ? (op & ~1ull) : op);
      const uint32_t i = o_start + (p - o_excl);
      // the slot's hit distance, infinity for a miss
      float t = __int_as_float(0x7f800000);
      if (act) {
        const float4 p0 = __ldg(P + 3 * i + 0);
        const float4 p1 = __ldg(P + 3 * i + 1);
        const float4 p2 = __ldg(P + 3 * i + 2);
        float th;
        // WT kernels serve watertight contexts, whose scenes all carry the exact vertices
        const bool hit = WT ? ray_tri_wt_body(p0, p1, p2, rx, ry, rz, sx, sy, sz, th)
                            : ray_tri(p0, p1, p2, rx, ry, rz, sx, sy, sz, th);
        if (hit) t = th;
      }
      // each owner takes its slots of this chunk in leaf order: the distance
      // from the slot's lane; its primitive (the owner's start + k) and that
      // primitive's surface and triangle ids the owner reads itself, for hits
      for (uint32_t k = 0; k < kmax; k++) {
        const uint32_t q = excl + k;
        const bool mine = own && k < cnt && q >= base && q < base + 32u;
        const uint32_t src = mine ? q - base : lane;
        const float tk = __shfl_sync(FULL, t, src);
        if (mine && tk < __int_as_float(0x7f800000)) {
          const uint32_t ik = start + k;
          const float* pw = reinterpret_cast<const float*>(lane_prims + 3 * ik);
          walk_take_tie(w, lane_prims, ik, tk, __float_as_uint(__ldg(pw + 11)), __float_as_uint(__ldg(pw + 7)));
        }
      }
    }
    __syncwarp();
    if (own && w.cur < 0) {
      w.leaf = w.cur;
      w.cur = walk_pop<true>(w);
    }
  }
}

}  // namespace

}  // namespace omg
