// Device routines shared by the tracer (trace.cu) and the dome (dome.cu):
// the per-ray stream, unit_sphere, normalize, the slab and Möller–Trumbore
// tests and the ordered closest-hit traversal. All f32 arithmetic follows the
// reference's operation order; the including files build with -fmad=false.
#pragma once
#include <cfloat>

#include "omg_internal.h"

namespace omg {

static constexpr float TAU_F = 6.28318530717958647692f;   // core::f32::consts::TAU
static constexpr float ONE_EPS = 1.0f + 1e-6f;              // mesh.rs:446,451 (f32 sum)

// Per-ray PCG-RXS-M-XS stream (trace_mesh.wgsl:90-98, seeding :211-213).
struct Pcg {
  uint32_t s;
  __device__ __forceinline__ void init(uint32_t seed, uint32_t ray) {
    s = (seed ^ (ray * 0x9E3779B9u)) + 1u;
    next();
    next();
  }
  __device__ __forceinline__ uint32_t next() {
    s = s * 747796405u + 2891336453u;
    uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (w >> 22u) ^ w;
  }
  // (x >> 8) / 2^24 (rng.rs:19-21 form); the product by 2^-24 is exact
  __device__ __forceinline__ float f32() { return (float)(next() >> 8u) * 5.9604644775390625e-8f; }
};

// sin and cos of an angle in [0, 2*pi], in f32 only: Cody-Waite reduction by
// pi/2 (pi/2 split in three f32 parts of 8, 11 and 24 significant bits, so the
// quadrant products are exact) and Taylor polynomials on [-pi/4, pi/4]
// (coefficients +-1/n!, Horner). Error within 3 ulp of the true values; the
// oracle evaluates the same operations in the same order, so both agree bit
// for bit.
__device__ __forceinline__ void sincos_f32(float phi, float& s, float& c) {
  const float k = rintf(phi * 0.636619772367581343f);
  const float r = ((phi - k * 1.5703125f) - k * 4.837512969970703125e-4f) - k * 7.54978995489188216e-8f;
  const float r2 = r * r;
  const float sp =
      r + r * r2 * (-1.66666666666666667e-1f +
                    r2 * (8.33333333333333333e-3f + r2 * (-1.98412698412698413e-4f + r2 * 2.75573192239858907e-6f)));
  const float cp =
      1.0f + r2 * (-0.5f + r2 * (4.16666666666666667e-2f +
                                 r2 * (-1.38888888888888889e-3f +
                                       r2 * (2.48015873015873016e-5f + r2 * -2.75573192239858907e-7f))));
  const int q = ((int)k) & 3;
  if (q == 0) { s = sp; c = cp; }
  else if (q == 1) { s = cp; c = -sp; }
  else if (q == 2) { s = -sp; c = -cp; }
  else { s = -cp; c = sp; }
}

// rng.rs:24-29
__device__ __forceinline__ void unit_sphere(Pcg& g, float& x, float& y, float& z) {
  float u1 = g.f32();
  z = 1.0f - 2.0f * u1;
  float r = sqrtf(fmaxf(1.0f - z * z, 0.0f));
  float phi = TAU_F * g.f32();
  float sf, cf;
  sincos_f32(phi, sf, cf);
  x = r * cf;
  y = r * sf;
}

// vec3.rs:19-26 (multiply by the reciprocal; (1,0,0) below 1e-12)
__device__ __forceinline__ void normalize3(float& x, float& y, float& z) {
  float l = sqrtf(x * x + y * y + z * z);
  if (l > 1e-12f) {
    float inv = __frcp_rn(l);  // IEEE 1/l, as 1.0f / l
    x = x * inv;
    y = y * inv;
    z = z * inv;
  } else {
    x = 1.0f;
    y = 0.0f;
    z = 0.0f;
  }
}

// mesh.rs:407-426. Swap by comparison (a NaN entry stays in place and fmaxf /
// fminf then ignore it, as Rust's f32::max/min do); the single final check is
// equivalent to the per-axis early exit because t0 only grows and t1 only
// shrinks.
__device__ __forceinline__ bool ray_aabb(float lx, float ly, float lz, float hx, float hy, float hz, float ox,
                                         float oy, float oz, float ix, float iy, float iz, float tmax, float& tout) {
  float t0 = 0.0f, t1 = tmax;
  float ta = (lx - ox) * ix, tb = (hx - ox) * ix;
  float lo = ta > tb ? tb : ta, hi = ta > tb ? ta : tb;
  t0 = fmaxf(t0, lo);
  t1 = fminf(t1, hi);
  ta = (ly - oy) * iy;
  tb = (hy - oy) * iy;
  lo = ta > tb ? tb : ta;
  hi = ta > tb ? ta : tb;
  t0 = fmaxf(t0, lo);
  t1 = fminf(t1, hi);
  ta = (lz - oz) * iz;
  tb = (hz - oz) * iz;
  lo = ta > tb ? tb : ta;
  hi = ta > tb ? ta : tb;
  t0 = fmaxf(t0, lo);
  t1 = fminf(t1, hi);
  tout = t0;
  return t0 <= t1;
}

// Slab test with t = fma(l, inv, -o inv) (oi = o inv) and min/max
// instructions, on boxes grown by DScene::nodes_f's margin. For an origin
// with |o_a| <= 7 M_a it accepts every box ray_aabb accepts on the ungrown
// box and returns an entry distance no larger: the rounding of t differs from
// ray_aabb's by at most 4 u (|lo_a| + |o_a|) |inv_a| <= 2^-22 8 M_a |inv_a|
// (u = 2^-24), no more than the margin 2^-19 M_a moves a face. It needs
// finite products: a direction component of 0 (inv infinite) can give
// inf - inf on one face and -inf on the other and close an axis the ray runs
// along, so walks with |d_a| < 2^-60 on any axis (or an origin beyond the
// margin) use ray_aabb on the grown boxes instead, which is exact for them
// and, the boxes being grown, accepts every box the ungrown test accepts.
// Used only where the visit order does not decide the hit (the near-tie
// rule), so the result is ray_aabb's.
__device__ __forceinline__ bool ray_aabb_fma(float lx, float ly, float lz, float hx, float hy, float hz, float oix,
                                             float oiy, float oiz, float ix, float iy, float iz, float tmax,
                                             float& tout) {
  const float ax = __fmaf_rn(lx, ix, -oix), bx = __fmaf_rn(hx, ix, -oix);
  const float ay = __fmaf_rn(ly, iy, -oiy), by = __fmaf_rn(hy, iy, -oiy);
  const float az = __fmaf_rn(lz, iz, -oiz), bz = __fmaf_rn(hz, iz, -oiz);
  const float t0 = fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fmaxf(fminf(az, bz), 0.0f));
  const float t1 = fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fminf(fmaxf(az, bz), tmax));
  tout = t0;
  return t0 <= t1;
}

// mesh.rs:436-456 — Möller–Trumbore, both faces, reference epsilons.
__device__ __forceinline__ bool ray_tri(const float4& p0, const float4& p1, const float4& p2, float ox, float oy,
                                        float oz, float dx, float dy, float dz, float& tout) {
  const float e1x = p1.x, e1y = p1.y, e1z = p1.z;
  const float e2x = p2.x, e2y = p2.y, e2z = p2.z;
  float px = dy * e2z - dz * e2y;
  float py = dz * e2x - dx * e2z;
  float pz = dx * e2y - dy * e2x;
  float det = e1x * px + e1y * py + e1z * pz;
  if (fabsf(det) < 1e-9f) return false;
  float inv = __frcp_rn(det);  // IEEE 1/det, as 1.0f / det
  float sx = ox - p0.x, sy = oy - p0.y, sz = oz - p0.z;
  float u = (sx * px + sy * py + sz * pz) * inv;
  if (!(u >= -1e-6f && u <= ONE_EPS)) return false;
  float qx = sy * e1z - sz * e1y;
  float qy = sz * e1x - sx * e1z;
  float qz = sx * e1y - sy * e1x;
  float v = (dx * qx + dy * qy + dz * qz) * inv;
  if (v < -1e-6f || u + v > ONE_EPS) return false;
  float t = (e2x * qx + e2y * qy + e2z * qz) * inv;
  if (t > 1e-5f) {
    tout = t;
    return true;
  }
  return false;
}

// Watertight ray-triangle test (Woop, Benthin, Wald 2013, "Watertight
// Ray/Triangle Intersection", JCGT 2(1)) on the exact vertices A, B, C (.xyz).
// The vertices are translated to the ray origin and sheared so that the ray
// runs along +z: kz is the axis of the largest |d_a| (the first of equal
// ones), kx and ky the next two, swapped when d_kz < 0 so that the winding
// stays. The signs of the 2D edge functions U, V, W decide the hit; an edge
// shared by two triangles gives both of them the same value with opposite
// signs (the same products of the same sheared coordinates), and a value that
// rounds to 0 is computed again in FP64 (exact products of f32 values), so a
// ray through a shared edge or vertex hits at least one of its triangles.
// Both faces count, and a hit needs t > 1e-5, as the reference's test
// (mesh.rs:455). Every step rounds as written (explicit round-to-nearest
// operations). ray_tri_wt is the out-of-line copy for walks that choose the
// test at run time; kernels compiled for watertight scenes inline the body.
__device__ __forceinline__ float pick3(float a, float b, float c, int k) { return k == 0 ? a : (k == 1 ? b : c); }

__device__ __forceinline__ bool ray_tri_wt_body(const float4 A4, const float4 B4, const float4 C4, float ox,
                                                float oy, float oz, float dx, float dy, float dz, float& tout) {
  const float adx = fabsf(dx), ady = fabsf(dy), adz = fabsf(dz);
  int kz = 0;
  if (ady > adx) kz = 1;
  if (adz > (kz == 0 ? adx : ady)) kz = 2;
  int kx = kz == 2 ? 0 : kz + 1;
  int ky = kx == 2 ? 0 : kx + 1;
  const float dkz = pick3(dx, dy, dz, kz);
  if (dkz < 0.0f) {
    const int k = kx;
    kx = ky;
    ky = k;
  }
  const float Sx = __fdiv_rn(pick3(dx, dy, dz, kx), dkz);
  const float Sy = __fdiv_rn(pick3(dx, dy, dz, ky), dkz);
  const float Sz = __fdiv_rn(1.0f, dkz);
  const float ax = __fsub_rn(A4.x, ox), ay = __fsub_rn(A4.y, oy), az = __fsub_rn(A4.z, oz);
  const float bx = __fsub_rn(B4.x, ox), by = __fsub_rn(B4.y, oy), bz = __fsub_rn(B4.z, oz);
  const float cx = __fsub_rn(C4.x, ox), cy = __fsub_rn(C4.y, oy), cz = __fsub_rn(C4.z, oz);
  const float akz = pick3(ax, ay, az, kz), bkz = pick3(bx, by, bz, kz), ckz = pick3(cx, cy, cz, kz);
  const float Ax = __fsub_rn(pick3(ax, ay, az, kx), __fmul_rn(Sx, akz));
  const float Ay = __fsub_rn(pick3(ax, ay, az, ky), __fmul_rn(Sy, akz));
  const float Bx = __fsub_rn(pick3(bx, by, bz, kx), __fmul_rn(Sx, bkz));
  const float By = __fsub_rn(pick3(bx, by, bz, ky), __fmul_rn(Sy, bkz));
  const float Cx = __fsub_rn(pick3(cx, cy, cz, kx), __fmul_rn(Sx, ckz));
  const float Cy = __fsub_rn(pick3(cx, cy, cz, ky), __fmul_rn(Sy, ckz));
  float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
  float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
  float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = __double2float_rn(__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx)));
    V = __double2float_rn(__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx)));
    W = __double2float_rn(__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax)));
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
  const float det = __fadd_rn(__fadd_rn(U, V), W);
  if (det == 0.0f) return false;
  const float Az = __fmul_rn(Sz, akz), Bz = __fmul_rn(Sz, bkz), Cz = __fmul_rn(Sz, ckz);
  const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
  const float t = __fdiv_rn(T, det);
  if (!(t > 1e-5f)) return false;
  tout = t;
  return true;
}

static __device__ __noinline__ bool ray_tri_wt(const float4 A4, const float4 B4, const float4 C4, float ox, float oy,
                                               float oz, float dx, float dy, float dz, float& tout) {
  return ray_tri_wt_body(A4, B4, C4, ox, oy, oz, dx, dy, dz, tout);
}

// The ray-triangle test of the closest-hit walks: the watertight test on the
// exact vertices (DScene::prims_wt) in watertight contexts (wt), else the
// reference's test on a, e1, e2 (DScene::prims).
__device__ __forceinline__ bool tri_hit(bool wt, const float4& p0, const float4& p1, const float4& p2, float ox,
                                        float oy, float oz, float dx, float dy, float dz, float& tout) {
  return wt ? ray_tri_wt(p0, p1, p2, ox, oy, oz, dx, dy, dz, tout)
            : ray_tri(p0, p1, p2, ox, oy, oz, dx, dy, dz, tout);
}

// mesh.rs:484-541 — ordered closest-hit traversal over the child-box BVH2.
// Visit order, culling (t_enter >= best) and the strict `<` on hits are the
// reference's, so over the reference tree the same triangle wins every tie.
//
// TIE = true resolves near-ties deterministically instead. Among all hits of
// the ray, let t_min be the nearest; every hit within t_min * (1 + 1e-6) is a
// near-tie of it, and the winner is the one of them with the lowest authored
// surface id, then original triangle id, then t. Coplanar copies of a shared
// wall, authored once per room with different materials, then resolve the
// same way at any precision (the rule segment_hits applies to crossings,
// mesh.rs:583-602). The winner depends only on the set of hits, so every
// tree, walk order and lane split finds the same one.
//
// A walk keeps, besides the winner so far, the exact t_min so far; nodes are
// culled beyond t_min * (1 + 1e-6). When a nearer hit shrinks the window so
// that the winner so far falls out of it while an earlier hit may still lie
// inside, the walk cannot know that hit any more: it flags `amb` and is then
// walked once more in `fixed` mode, with the final window, taking the lowest
// key among the hits inside it. That second walk is rare (three hits within
// about 1e-6 of each other) and short (everything beyond the window is culled).
constexpr float kTieRel = 1e-6f;

struct TieState {
  float t_min;   // nearest hit so far (FLT_MAX: none)
  bool amb;      // the window shrank past a hit this walk no longer knows
  bool fixed;    // second walk: the window is final (t_cull), take the lowest key in it
};

__device__ __forceinline__ TieState tie_begin() {
  TieState z;
  z.t_min = FLT_MAX;
  z.amb = false;
  z.fixed = false;
  return z;
}

// (surface, triangle, t) of a below (s, tr, t) of b
__device__ __forceinline__ bool tie_key_less(uint32_t as, uint32_t atr, float at, uint32_t bs, uint32_t btr, float bt) {
  return as < bs || (as == bs && (atr < btr || (atr == btr && at < bt)));
}

// One hit (t, surface s, triangle tr) into a near-tie walk's state; true when
// it becomes the winner so far. t_cull follows the window.
__device__ __forceinline__ bool tie_take(float t, uint32_t s, uint32_t tr, bool have, float t_best, float& t_cull,
                                         uint32_t s_best, uint32_t tri_best, TieState& ts) {
  bool take;
  if (ts.fixed) {
    take = t <= t_cull && (!have || tie_key_less(s, tr, t, s_best, tri_best, t_best));
  } else if (!have) {
    take = true;
    ts.t_min = t;
  } else if (t < ts.t_min) {
    const float win = t * (1.0f + kTieRel);
    if (t_best <= win) {
      take = tie_key_less(s, tr, t, s_best, tri_best, t_best);
    } else {
      if (ts.t_min <= win) ts.amb = true;
      take = true;
    }
    ts.t_min = t;
  } else {
    take = t <= t_cull && tie_key_less(s, tr, t, s_best, tri_best, t_best);
  }
  if (!ts.fixed) t_cull = ts.t_min * (1.0f + kTieRel);
  return take;
}

template <bool TIE>
__device__ __forceinline__ bool leaf_test(const float4* __restrict__ prims, int leaf, float ox, float oy, float oz,
                                          float dx, float dy, float dz, bool& have, float& t_best, float& t_cull,
                                          int& prim_best, uint32_t& s_best, uint32_t& tri_best, TieState& ts,
                                          bool wt = false) {
  const uint32_t code = ~(uint32_t)leaf;
  const uint32_t start = code >> 3, end = start + (code & 7u) + 1u;
  for (uint32_t i = start; i < end; i++) {
    const float4 p0 = __ldg(prims + 3 * i + 0);
    const float4 p1 = __ldg(prims + 3 * i + 1);
    const float4 p2 = __ldg(prims + 3 * i + 2);
    float t;
    if (tri_hit(wt, p0, p1, p2, ox, oy, oz, dx, dy, dz, t)) {
      if (!TIE) {
        if (!have || t < t_best) {
          have = true;
          t_best = t;
          prim_best = (int)i;
          t_cull = t;
        }
      } else {
        const uint32_t s = __float_as_uint(p2.w), tr = __float_as_uint(p1.w);
        if (tie_take(t, s, tr, have, t_best, t_cull, s_best, tri_best, ts)) {
          have = true;
          t_best = t;
          prim_best = (int)i;
          s_best = s;
          tri_best = tr;
        }
      }
    }
  }
  return have;
}

// While-while traversal (Aila & Laine 2009). With TIE the traversal is
// speculative: a lane that reaches a leaf postpones it and keeps descending
// until every active lane of the warp holds a leaf, so triangle tests run
// together; the nearest hit is the same (only culling is later), and the
// tie rule makes the winner independent of the visit order. Without TIE a
// leaf is tested as soon as it is reached: the reference's exact order.
template <bool TIE>
__device__ __forceinline__ bool mesh_closest(const DScene& S, float ox, float oy, float oz, float dx, float dy,
                                             float dz, float& t_best, int& prim_best, uint32_t* err) {
  if (S.n_prims == 0) return false;
  constexpr int kDone = 0x7FFFFFFF;  // never a node index (< 2^28)
  const float ix = __frcp_rn(dx), iy = __frcp_rn(dy), iz = __frcp_rn(dz);
  // near-tie walks use the grown boxes (DScene::nodes_f): they find every hit
  // of every primitive, whatever the tree (the exact test on them)
  const float4* __restrict__ nodes = (TIE && S.nodes_f) ? S.nodes_f : S.nodes;
  const bool wt = S.prims_wt != nullptr;
  const float4* __restrict__ prims = wt ? S.prims_wt : S.prims;
  bool have = false;
  t_best = FLT_MAX;
  float t_cull = FLT_MAX;            // TIE: t_min * (1 + 1e-6); else best; FLT_MAX before the first hit
  uint32_t s_best = 0, tri_best = 0;
  TieState ts = tie_begin();
  int stack_ref[STACK_DEPTH];
  float stack_t[STACK_DEPTH];
  int sp = 0;
  int cur = S.root;
  int leaf = 0;                      // postponed leaf (< 0), or 0
  // every node and leaf is visited at most once per ray and pass: a walk
  // longer than this bound means a corrupt tree; stop and flag it rather than spin
  uint32_t budget = S.walk_budget;
  auto culled = [&](float t) { return TIE ? t > t_cull : (have && t >= t_best); };
  // next stacked entry that is not culled, or kDone
  auto pop = [&]() -> int {
    while (sp > 0) {
      sp--;
      if (culled(stack_t[sp])) continue;
      return stack_ref[sp];
    }
    return kDone;
  };
  while (true) {
    while (cur != kDone || leaf < 0) {
      // ---- internal nodes
      while (cur >= 0 && cur != kDone) {
        if (budget-- == 0u) {
          atomicOr(err, 4u);
          return have;
        }
        const float4 n0 = __ldg(nodes + 4 * cur + 0);
        const float4 n1 = __ldg(nodes + 4 * cur + 1);
        const float4 n2 = __ldg(nodes + 4 * cur + 2);
        const float4 n3 = __ldg(nodes + 4 * cur + 3);
        const float tmax = t_cull;
        float ta, tb;
        const bool h0 = ray_aabb(n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, ox, oy, oz, ix, iy, iz, tmax, ta);
        const bool h1 = ray_aabb(n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, ox, oy, oz, ix, iy, iz, tmax, tb);
        const int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
        if (h0 && h1) {
          int nr, fr;
          float nt, ft;
          if (ta <= tb) { nr = c0; nt = ta; fr = c1; ft = tb; }
          else { nr = c1; nt = tb; fr = c0; ft = ta; }
          if (sp < STACK_DEPTH) {
            stack_ref[sp] = fr;
            stack_t[sp] = ft;
            sp++;
          } else {
            atomicOr(err, 1u);
          }
          cur = culled(nt) ? pop() : nr;
        } else if (h0) {
          cur = culled(ta) ? pop() : c0;
        } else if (h1) {
          cur = culled(tb) ? pop() : c1;
        } else {
          cur = pop();
        }
        if (TIE) {
          if (cur < 0 && leaf == 0) {  // postpone the leaf, keep descending
            leaf = cur;
            cur = pop();
          }
          if (__all_sync(__activemask(), leaf < 0 || cur == kDone)) break;
        }
      }
      // ---- leaves (the postponed one, then any leaf the stack yields next)
      if (!TIE) {
        if (cur == kDone) break;
        if (budget-- == 0u) {
          atomicOr(err, 4u);
          return have;
        }
        leaf_test<TIE>(prims, cur, ox, oy, oz, dx, dy, dz, have, t_best, t_cull, prim_best, s_best, tri_best, ts,
                       wt);
        cur = pop();
      } else {
        if (leaf == 0 && cur < 0) {  // a leaf reached outside the node loop (e.g. a leaf root)
          leaf = cur;
          cur = pop();
        }
        while (leaf < 0) {
          if (budget-- == 0u) {
            atomicOr(err, 4u);
            return have;
          }
          leaf_test<TIE>(prims, leaf, ox, oy, oz, dx, dy, dz, have, t_best, t_cull, prim_best, s_best, tri_best,
                         ts, wt);
          leaf = 0;
          if (cur < 0) {
            leaf = cur;
            cur = pop();
          }
        }
      }
    }
    if (!TIE || !ts.amb || ts.fixed) break;
    // the near-tie window shrank past a hit this walk no longer knows: walk
    // once more with the final window
    ts.fixed = true;
    t_cull = ts.t_min * (1.0f + kTieRel);
    have = false;
    t_best = FLT_MAX;
    sp = 0;
    cur = S.root;
    leaf = 0;
    budget = S.walk_budget;
  }
  return have;
}

// Closest hit with the near-tie rule (TIE = true above) over the 4-wide tree
// (DScene::nodes4). A node step tests the 4 child boxes, tests the hit leaf
// children at once and descends into the nearest hit internal child, pushing
// the others farthest first. Because the tie rule makes the winner
// independent of the visit order and a box is skipped only beyond
// the window, the hit is the one the binary walk finds: the near-tie rule
// depends only on the set of hits (TieState).
//
// One node step; returns the next node, or kDone4 once the stack is empty.
constexpr int kDone4 = 0x7FFFFFFF;
__device__ __forceinline__ int bvh4_step(const float4* __restrict__ nodes, const float4* __restrict__ prims, int cur,
                                         float ox, float oy, float oz, float dx, float dy, float dz, float ix,
                                         float iy, float iz, bool& have, float& t_best, float& t_cull,
                                         int& prim_best, uint32_t& s_best, uint32_t& tri_best, TieState& ts,
                                         int* stack_ref, float* stack_t, int& sp, uint32_t* err, bool wt = false) {
  const float4* nd = nodes + 8 * cur;
  const float4 lx = __ldg(nd + 0), hx = __ldg(nd + 1), ly = __ldg(nd + 2), hy = __ldg(nd + 3);
  const float4 lz = __ldg(nd + 4), hz = __ldg(nd + 5), rf = __ldg(nd + 6);
  const float tmax = t_cull;
  const float blx[4] = {lx.x, lx.y, lx.z, lx.w}, bhx[4] = {hx.x, hx.y, hx.z, hx.w};
  const float bly[4] = {ly.x, ly.y, ly.z, ly.w}, bhy[4] = {hy.x, hy.y, hy.z, hy.w};
  const float blz[4] = {lz.x, lz.y, lz.z, lz.w}, bhz[4] = {hz.x, hz.y, hz.z, hz.w};
  const int ref[4] = {__float_as_int(rf.x), __float_as_int(rf.y), __float_as_int(rf.z), __float_as_int(rf.w)};
  float t[4];
  int r[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    float tk;
    const bool h = ref[k] != kEmpty4 &&
                   ray_aabb(blx[k], bly[k], blz[k], bhx[k], bhy[k], bhz[k], ox, oy, oz, ix, iy, iz, tmax, tk);
    t[k] = h ? tk : FLT_MAX;
    r[k] = h ? ref[k] : kDone4;
  }
  // leaves first, nearest first
#pragma unroll
  for (int k = 0; k < 4; k++) {
    int bk = -1;
    float bt = FLT_MAX;
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (r[j] < 0 && t[j] <= bt) { bt = t[j]; bk = j; }
    if (bk < 0) break;
    if (bt <= t_cull)
      leaf_test<true>(prims, r[bk], ox, oy, oz, dx, dy, dz, have, t_best, t_cull, prim_best, s_best, tri_best, ts,
                      wt);
    r[bk] = kDone4;
    t[bk] = FLT_MAX;
  }
  // internal children by entry distance (sorting network): the nearest is
  // the next node, the others are pushed farthest first
  auto cswap = [&](int a, int b) {
    if (t[b] < t[a]) {
      const float tt = t[a]; t[a] = t[b]; t[b] = tt;
      const int rr = r[a]; r[a] = r[b]; r[b] = rr;
    }
  };
  cswap(0, 1); cswap(2, 3); cswap(0, 2); cswap(1, 3); cswap(1, 2);
#pragma unroll
  for (int k = 3; k >= 1; k--) {
    if (r[k] == kDone4 || t[k] > t_cull) continue;
    if (sp < STACK_DEPTH) { stack_ref[sp] = r[k]; stack_t[sp] = t[k]; sp++; }
    else atomicOr(err, 1u);
  }
  int nxt = (r[0] == kDone4 || t[0] > t_cull) ? kDone4 : r[0];
  while (nxt == kDone4 && sp > 0) {
    sp--;
    if (stack_t[sp] > t_cull) continue;
    nxt = stack_ref[sp];
  }
  return nxt;
}

__device__ __forceinline__ bool mesh_closest4(const DScene& S, float ox, float oy, float oz, float dx, float dy,
                                              float dz, float& t_best, int& prim_best, uint32_t* err) {
  t_best = FLT_MAX;
  if (S.n_prims == 0) return false;
  const float ix = __frcp_rn(dx), iy = __frcp_rn(dy), iz = __frcp_rn(dz);
  bool have = false;
  float t_cull = FLT_MAX;
  uint32_t s_best = 0, tri_best = 0;
  TieState ts = tie_begin();
  int stack_ref[STACK_DEPTH];
  float stack_t[STACK_DEPTH];
  int sp = 0;
  int cur = S.root4;
  uint32_t budget = S.walk_budget4;   // every node is entered at most once per pass
  while (true) {
    while (cur != kDone4) {
      if (budget-- == 0u) {
        atomicOr(err, 4u);
        return have;
      }
      cur = bvh4_step(S.nodes4, S.prims_wt ? S.prims_wt : S.prims, cur, ox, oy, oz, dx, dy, dz, ix, iy, iz, have,
                      t_best, t_cull, prim_best, s_best, tri_best, ts, stack_ref, stack_t, sp, err,
                      S.prims_wt != nullptr);
    }
    if (!ts.amb || ts.fixed) break;
    // a second walk with the final near-tie window (see TieState)
    ts.fixed = true;
    t_cull = ts.t_min * (1.0f + kTieRel);
    have = false;
    t_best = FLT_MAX;
    sp = 0;
    cur = S.root4;
    budget = S.walk_budget4;
  }
  return have;
}

}  // namespace omg
