// World early reflections on the GPU (crates/omg-core/src/pt_mesh.rs).
//
// Discovery (mesh_chains, pt_mesh.rs:382-457): one thread per fan ray bounces
// specularly off the mesh and the furniture boxes up to 3 times; every
// surface chain it passes is a candidate. A global hash table keeps, per
// chain, the lowest candidate index (ray-major, bounce-minor: the order in
// which the reference's sequential loop meets them), and one block compacts
// the first occurrences in that order, which is the reference's output order.
//
// Solve (mesh_record, pt_mesh.rs:186-337): one thread per (source, chain)
// pair mirrors the source across the chain's planes, validates each bounce by
// a closest-hit query (the reference's first-found order over the binary
// tree) and pays the transmission of every surface and blocker each leg
// crosses (segment_hits, mesh.rs:546-604: crossings in depth-first order,
// stably sorted by t, equal-t clusters merged to the lowest surface id).
//
// f32 arithmetic in the reference's operation order (built with -fmad=false,
// IEEE division and square root); cos/sin of the fan azimuth and exp of the
// air attenuation are evaluated in double and rounded once.
#include <cfloat>

#include "device_common.cuh"

namespace omg {

namespace {

constexpr uint16_t kNoSurf = 0xFFFFu;
constexpr uint32_t kMaxSeg = 64;             // crossings kept per segment query

__device__ __forceinline__ float dot3(const float a[3], float x, float y, float z) {
  return a[0] * x + a[1] * y + a[2] * z;
}

__device__ __forceinline__ float len3(float x, float y, float z) { return sqrtf(x * x + y * y + z * z); }

__device__ __forceinline__ bool dead3(const float v[3], float lim) { return v[0] < lim && v[1] < lim && v[2] < lim; }

// Closest hit in the reference's first-found order: (t, original triangle,
// material) or false.
__device__ __forceinline__ bool raycast_ref(const DEarly& E, float ox, float oy, float oz, float dx, float dy,
                                            float dz, float& t, uint32_t& tri, uint32_t& mat) {
  int prim = 0;
  if (!mesh_closest<false>(E.S, ox, oy, oz, dx, dy, dz, t, prim, E.err)) return false;
  mat = __float_as_uint(__ldg(E.S.prims + 3 * prim + 0).w);
  tri = __float_as_uint(__ldg(E.S.prims + 3 * prim + 1).w);
  return true;
}

// ------------------------------------------------------------- discovery
struct DiscArgs {
  DEarly E;
  float lx, ly, lz;
  uint32_t n_rays, rot;
  uint32_t use_boxes;
  float ga;                           // golden angle, f32 (pt_mesh.rs:392)
  const float* jitter;                // the rotation's xorshift draws, one per ray
  unsigned long long* cand_key;
  omg_chain* cand_chain;
  uint32_t* cand_slot;
  unsigned long long* tkey;
  uint32_t* tidx;
  uint32_t tcap;
};

__device__ __forceinline__ uint32_t key_hash(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  return (uint32_t)k;
}

__global__ void early_discover_kernel(DiscArgs A) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.n_rays) return;
  const DEarly& E = A.E;
  for (int k = 0; k < OMG_CHAIN_MAX_ORDER; k++) A.cand_key[3 * i + k] = 0ull;
  const float z = 1.0f - 2.0f * ((float)i + 0.5f) / (float)A.n_rays;
  const float r = sqrtf(fmaxf(1.0f - z * z, 0.0f));
  const float phi = A.ga * (float)i + (float)A.rot * 0.61803398875f * 6.28318530717958647692f + A.jitter[i] * 0.02f;
  double sd, cd;
  sincos((double)phi, &sd, &cd);
  float dx = r * (float)cd, dy = r * (float)sd, dz = z;
  float px = A.lx, py = A.ly, pz = A.lz;
  uint16_t chain[OMG_CHAIN_MAX_ORDER] = {kNoSurf, kNoSurf, kNoSurf};
  for (int k = 0; k < OMG_CHAIN_MAX_ORDER; k++) {
    float t = FLT_MAX, nx = 0.0f, ny = 0.0f, nz = 1.0f;
    bool has = false;
    uint32_t sid = 0;
    {
      float mt;
      uint32_t tri, mat;
      if (raycast_ref(E, px, py, pz, dx, dy, dz, mt, tri, mat)) {
        t = mt;
        has = true;
        sid = E.S.tri_surface[tri];
        const float4 nn = __ldg(E.S.normals + tri);
        nx = nn.x;
        ny = nn.y;
        nz = nn.z;
      }
    }
    if (A.use_boxes) {
      const float p[3] = {px, py, pz}, d[3] = {dx, dy, dz};
      for (uint32_t bi = 0; bi < E.n_boxes; bi++) {
        const float4 bl = __ldg(E.boxes + 2 * bi), bh = __ldg(E.boxes + 2 * bi + 1);
        const float mn[3] = {bl.x, bl.y, bl.z}, mx[3] = {bh.x, bh.y, bh.z};
        float t0 = 1e-4f, t1 = t;
        int axis = 3;
        for (int a = 0; a < 3; a++) {
          const float da = d[a];
          if (fabsf(da) < 1e-9f) {
            if (p[a] < mn[a] || p[a] > mx[a]) {
              t0 = FLT_MAX;
              break;
            }
          } else {
            float ta = (mn[a] - p[a]) / da, tb = (mx[a] - p[a]) / da;
            if (ta > tb) {
              const float q = ta;
              ta = tb;
              tb = q;
            }
            if (ta > t0) {
              t0 = ta;
              axis = a;
            }
            t1 = fminf(t1, tb);
            if (t0 > t1) {
              t0 = FLT_MAX;
              break;
            }
          }
        }
        if (t0 < t && axis < 3) {
          t = t0;
          const int face = axis * 2 + (d[axis] > 0.0f ? 0 : 1);
          has = true;
          sid = (E.base_overlay + bi * 6u + (uint32_t)face) & 0xFFFFu;
          nx = ny = nz = 0.0f;
          const float s = d[axis] > 0.0f ? -1.0f : 1.0f;
          if (axis == 0) nx = s;
          else if (axis == 1) ny = s;
          else nz = s;
        }
      }
    }
    if (!has) break;
    if (t <= 1e-4f || t > 200.0f) break;
    px = px + dx * t;
    py = py + dy * t;
    pz = pz + dz * t;
    chain[k] = (uint16_t)sid;
    unsigned long long key = 1ull;
    for (int q = 0; q <= k; q++) key = key * 65536ull + (unsigned long long)chain[q] + 1ull;
    const uint32_t j = 3u * i + (uint32_t)k;
    A.cand_key[j] = key;
    omg_chain c;
    for (int q = 0; q < OMG_CHAIN_MAX_ORDER; q++) c.surf[q] = chain[q];
    c.order = (uint16_t)(k + 1);
    A.cand_chain[j] = c;
    // first occurrence per key: the lowest candidate index
    uint32_t h = key_hash(key) & (A.tcap - 1u);
    bool placed = false;
    for (uint32_t probe = 0; probe < A.tcap; probe++) {
      const unsigned long long prev = atomicCAS(A.tkey + h, 0ull, key);
      if (prev == 0ull || prev == key) {
        atomicMin(A.tidx + h, j);
        A.cand_slot[j] = h;
        placed = true;
        break;
      }
      h = (h + 1u) & (A.tcap - 1u);
    }
    if (!placed) {
      atomicOr(E.err, 8u);
      A.cand_key[j] = 0ull;
    }
    // specular bounce off the hit normal, faced against the ray
    const float dn0 = nx * dx + ny * dy + nz * dz;
    if (dn0 > 0.0f) {
      nx = nx * -1.0f;
      ny = ny * -1.0f;
      nz = nz * -1.0f;
    }
    const float s2 = 2.0f * (dx * nx + dy * ny + dz * nz);
    dx = dx - nx * s2;
    dy = dy - ny * s2;
    dz = dz - nz * s2;
    px = px + nx * 1e-4f;
    py = py + ny * 1e-4f;
    pz = pz + nz * 1e-4f;
  }
}

// One block: the first occurrences, compacted in candidate order.
constexpr uint32_t kCompactThreads = 1024;
__global__ void __launch_bounds__(kCompactThreads)
    early_compact_kernel(const unsigned long long* __restrict__ cand_key, const omg_chain* __restrict__ cand_chain,
                         const uint32_t* __restrict__ cand_slot, const uint32_t* __restrict__ tidx, uint32_t n_cand,
                         omg_chain* out, uint32_t cap, uint32_t* n_out) {
  __shared__ uint32_t warp_tot[kCompactThreads / 32];
  __shared__ uint32_t base;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  if (tid == 0) base = 0;
  __syncthreads();
  for (uint32_t chunk = 0; chunk < n_cand; chunk += kCompactThreads) {
    const uint32_t j = chunk + tid;
    const bool keep = j < n_cand && cand_key[j] != 0ull && tidx[cand_slot[j]] == j;
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) warp_tot[warp] = (uint32_t)__popc(m);
    __syncthreads();
    if (warp == 0) {
      const uint32_t v = warp_tot[lane];
      uint32_t incl = v;
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += u;
      }
      warp_tot[lane] = incl - v;   // exclusive prefix of the warps
    }
    __syncthreads();
    const uint32_t pos = base + warp_tot[warp] + (uint32_t)__popc(m & ((1u << lane) - 1u));
    if (keep && pos < cap) out[pos] = cand_chain[j];
    __syncthreads();
    if (tid == kCompactThreads - 1) base = pos + (keep ? 1u : 0u);
    __syncthreads();
  }
  if (tid == 0) *n_out = base;
}

// ----------------------------------------------------------------- solve
struct SegList {
  float t[kMaxSeg];
  uint32_t tri[kMaxSeg];
  uint32_t mat[kMaxSeg];
  uint32_t n;
};

// mesh.rs:546-604 — every crossing of a->b strictly between its ends, in the
// reference's order, merged.
__device__ void segment_hits(const DEarly& E, float ax, float ay, float az, float bx, float by, float bz, SegList& L) {
  L.n = 0;
  const DScene& S = E.S;
  if (S.n_prims == 0) return;
  float dx = bx - ax, dy = by - ay, dz = bz - az;
  const float len = len3(dx, dy, dz);
  if (len < 1e-6f) return;
  const float il = __frcp_rn(len);
  dx = dx * il;
  dy = dy * il;
  dz = dz * il;
  const float ix = __frcp_rn(dx), iy = __frcp_rn(dy), iz = __frcp_rn(dz);
  float tr;
  if (!ray_aabb(E.root_lo[0], E.root_lo[1], E.root_lo[2], E.root_hi[0], E.root_hi[1], E.root_hi[2], ax, ay, az, ix,
                iy, iz, len, tr))
    return;
  int stack[STACK_DEPTH];
  int sp = 0;
  stack[sp++] = S.root;
  uint32_t budget = S.walk_budget;
  bool full = false;
  while (sp > 0) {
    if (budget-- == 0u) {
      atomicOr(E.err, 4u);
      break;
    }
    const int cur = stack[--sp];
    if (cur >= 0) {
      const float4 n0 = __ldg(S.nodes + 4 * cur + 0);
      const float4 n1 = __ldg(S.nodes + 4 * cur + 1);
      const float4 n2 = __ldg(S.nodes + 4 * cur + 2);
      const float4 n3 = __ldg(S.nodes + 4 * cur + 3);
      float ta, tb;
      const bool h0 = ray_aabb(n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, ax, ay, az, ix, iy, iz, len, ta);
      const bool h1 = ray_aabb(n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, ax, ay, az, ix, iy, iz, len, tb);
      // the reference pushes a then b and pops b first
      if (h0) {
        if (sp < STACK_DEPTH) stack[sp++] = __float_as_int(n3.x);
        else atomicOr(E.err, 1u);
      }
      if (h1) {
        if (sp < STACK_DEPTH) stack[sp++] = __float_as_int(n3.y);
        else atomicOr(E.err, 1u);
      }
    } else {
      const uint32_t code = ~(uint32_t)cur;
      const uint32_t start = code >> 3, end = start + (code & 7u) + 1u;
      for (uint32_t i = start; i < end; i++) {
        const float4 p0 = __ldg(S.prims + 3 * i + 0);
        const float4 p1 = __ldg(S.prims + 3 * i + 1);
        const float4 p2 = __ldg(S.prims + 3 * i + 2);
        float t;
        if (ray_tri(p0, p1, p2, ax, ay, az, dx, dy, dz, t)) {
          const float tt = t / len;
          if (tt > 1e-4f && tt < 1.0f - 1e-4f) {
            if (L.n < kMaxSeg) {
              // stable insertion by t (crossings arrive in depth-first order)
              uint32_t q = L.n;
              while (q > 0 && L.t[q - 1] > tt) {
                L.t[q] = L.t[q - 1];
                L.tri[q] = L.tri[q - 1];
                L.mat[q] = L.mat[q - 1];
                q--;
              }
              L.t[q] = tt;
              L.tri[q] = __float_as_uint(p1.w);
              L.mat[q] = __float_as_uint(p0.w);
              L.n++;
            } else {
              full = true;
            }
          }
        }
      }
    }
  }
  if (full) atomicOr(E.err, 2u);
  // same-t clusters: the lowest surface id wins, the cluster keeps its first t
  const float tol = 1e-4f / fmaxf(len, 1.0f);
  uint32_t w = 0;
  for (uint32_t i = 0; i < L.n; i++) {
    if (w > 0 && fabsf(L.t[i] - L.t[w - 1]) < tol) {
      if (S.tri_surface[L.tri[i]] < S.tri_surface[L.tri[w - 1]]) {
        L.tri[w - 1] = L.tri[i];
        L.mat[w - 1] = L.mat[i];
      }
    } else {
      L.t[w] = L.t[i];
      L.tri[w] = L.tri[i];
      L.mat[w] = L.mat[i];
      w++;
    }
  }
  L.n = w;
}

// pt.rs:43-70
__device__ __forceinline__ bool aabb_clip(const omg_aabb& x, float ax, float ay, float az, float bx, float by,
                                          float bz) {
  const float a[3] = {ax, ay, az}, d[3] = {bx - ax, by - ay, bz - az};
  float t0 = 0.0f, t1 = 1.0f;
  for (int k = 0; k < 3; k++) {
    if (fabsf(d[k]) < 1e-9f) {
      if (a[k] < x.mn[k] || a[k] > x.mx[k]) return false;
    } else {
      float ta = (x.mn[k] - a[k]) / d[k], tb = (x.mx[k] - a[k]) / d[k];
      if (ta > tb) {
        const float q = ta;
        ta = tb;
        tb = q;
      }
      t0 = fmaxf(t0, ta);
      t1 = fminf(t1, tb);
      if (t0 > t1) return false;
    }
  }
  return t1 > 1e-4f && t0 < 1.0f - 1e-4f;
}

// pt_mesh.rs:146-182
__device__ bool leg_transmission(const DEarly& E, float ax, float ay, float az, float bx, float by, float bz,
                                 bool has_skip, uint32_t skip_sid, float t_expect, const omg_aabb* extras,
                                 uint32_t n_extras, SegList& L, float tr[3]) {
  segment_hits(E, ax, ay, az, bx, by, bz, L);
  const float seg_len = fmaxf(len3(bx - ax, by - ay, bz - az), 1e-6f);
  for (uint32_t i = 0; i < L.n; i++) {
    if (has_skip && E.S.tri_surface[L.tri[i]] == skip_sid && fabsf(L.t[i] - t_expect) * seg_len < 0.05f) continue;
    const float4 m = __ldg(E.mtrans + L.mat[i]);
    tr[0] = tr[0] * m.x;
    tr[1] = tr[1] * m.y;
    tr[2] = tr[2] * m.z;
    if (dead3(tr, 1e-6f)) return false;
  }
  for (uint32_t k = 0; k < n_extras; k++) {
    if (aabb_clip(extras[k], ax, ay, az, bx, by, bz)) {
      for (int b = 0; b < 3; b++) tr[b] = tr[b] * extras[k].transmission[b];
      if (dead3(tr, 1e-6f)) return false;
    }
  }
  return true;
}

// pt_mesh.rs:186-337
__device__ bool mesh_record(const DEarly& E, const omg_chain& ch, uint16_t source, float sx, float sy, float sz,
                            float lx, float ly, float lz, const omg_aabb* extras, uint32_t n_extras, SegList& L,
                            omg_mesh_record& out) {
  const int order = ch.order;
  float ix = sx, iy = sy, iz = sz;
  for (int i = order - 1; i >= 0; i--) {
    if (ch.surf[i] >= E.n_surf) return false;
    const DSurf& s = E.surf[ch.surf[i]];
    const float k = 2.0f * (dot3(s.n, ix, iy, iz) - s.d);
    ix = ix - s.n[0] * k;
    iy = iy - s.n[1] * k;
    iz = iz - s.n[2] * k;
  }
  const float tx = ix - lx, ty = iy - ly, tz = iz - lz;
  const float dist = len3(tx, ty, tz);
  if (dist < 1e-4f) return false;
  const float idist = __frcp_rn(dist);
  const float dirx = tx * idist, diry = ty * idist, dirz = tz * idist;
  float gm[3] = {1.0f, 1.0f, 1.0f};
  float px = lx, py = ly, pz = lz, dx = dirx, dy = diry, dz = dirz;
  for (int i = 0; i < order; i++) {
    const uint32_t sid = ch.surf[i];
    if (sid >= E.n_surf) return false;
    const DSurf& s = E.surf[sid];
    const float denom = dot3(s.n, dx, dy, dz);
    if (fabsf(denom) < 1e-9f) return false;
    const float t = (s.d - dot3(s.n, px, py, pz)) / denom;
    if (t <= 1e-4f) return false;
    const float hx = px + dx * t, hy = py + dy * t, hz = pz + dz * t;
    const float ox = px + dx * 1e-4f, oy = py + dy * 1e-4f, oz = pz + dz * 1e-4f;
    float rt;
    uint32_t rtri, rmat;
    if (s.rect) {
      const float eps = 1e-3f;
      const float h[3] = {hx, hy, hz};
      for (int a = 0; a < 3; a++)
        if (h[a] < s.fmin[a] - eps || h[a] > s.fmax[a] + eps) return false;
      if (raycast_ref(E, ox, oy, oz, dx, dy, dz, rt, rtri, rmat) && rt < t - 1e-3f) {
        const float4 m = __ldg(E.mtrans + rmat);
        const float mt[3] = {m.x, m.y, m.z};
        if (dead3(mt, 1e-6f)) return false;
      }
    } else {
      if (!raycast_ref(E, ox, oy, oz, dx, dy, dz, rt, rtri, rmat)) return false;
      const bool on_surface = E.S.tri_surface[rtri] == sid && fabsf(rt - t) < 2e-2f;
      if (!on_surface) {
        if (rt < t - 1e-3f) {
          const float4 m = __ldg(E.mtrans + rmat);
          const float mt[3] = {m.x, m.y, m.z};
          if (dead3(mt, 1e-4f)) return false;
          segment_hits(E, px, py, pz, hx + dx * 0.05f, hy + dy * 0.05f, hz + dz * 0.05f, L);
          bool found = false;
          for (uint32_t q = 0; q < L.n; q++)
            if (E.S.tri_surface[L.tri[q]] == sid && fabsf(L.t[q] * (t + 0.05f) - t) < 0.1f) found = true;
          if (!found) return false;
        } else {
          return false;
        }
      }
    }
    if (!leg_transmission(E, px, py, pz, hx, hy, hz, true, sid, 1.0f, extras, n_extras, L, gm)) return false;
    for (int b = 0; b < 3; b++) gm[b] = gm[b] * s.refl[b];
    const float nd = dot3(s.n, dx, dy, dz);
    const float off = nd < 0.0f ? 1e-4f : -1e-4f;
    px = hx + s.n[0] * off;
    py = hy + s.n[1] * off;
    pz = hz + s.n[2] * off;
    const float k2 = 2.0f * nd;
    dx = dx - s.n[0] * k2;
    dy = dy - s.n[1] * k2;
    dz = dz - s.n[2] * k2;
  }
  if (order > 0) {
    const DSurf& s = E.surf[ch.surf[order - 1]];
    if ((dot3(s.n, px, py, pz) - s.d) * (dot3(s.n, sx, sy, sz) - s.d) < 0.0f) return false;
  }
  if (!leg_transmission(E, px, py, pz, sx, sy, sz, false, 0u, 0.0f, extras, n_extras, L, gm)) return false;
  if (order > 0) {
    const float qx = sx - px, qy = sy - py, qz = sz - pz;
    const float leg = len3(qx, qy, qz);
    if (leg > 1e-4f) {
      const float il = __frcp_rn(leg);
      if ((qx * il) * dx + (qy * il) * dy + (qz * il) * dz < 0.995f) return false;
    }
  }
  const float dtot = fmaxf(dist, 0.3f);
  const float kAir[3] = {1.0e-4f, 5.0e-4f, 3.0e-3f};  // AIR_ABSORPTION_PER_M, material.rs:76
  float gains[3];
  for (int b = 0; b < 3; b++) {
    const float air = (float)exp((double)(-kAir[b] * dtot));
    gains[b] = air / dtot * gm[b];
  }
  if (dead3(gains, 2e-5f)) return false;
  out.source = source;
  for (int q = 0; q < OMG_CHAIN_MAX_ORDER; q++) out.chain[q] = q < order ? ch.surf[q] : kNoSurf;
  out.order = (uint32_t)order;
  out.delay_s = dist / 343.0f;
  out.dir[0] = dirx;
  out.dir[1] = diry;
  out.dir[2] = dirz;
  for (int b = 0; b < 3; b++) out.gains[b] = gains[b];
  uint32_t h = 0x811C9DC5u ^ (uint32_t)source;
  for (int q = 0; q < order; q++) h = (h ^ (uint32_t)ch.surf[q]) * 16777619u;
  out.key = (h ^ 0xA5u) * 16777619u;
  out.valid = 1u;
  return true;
}

struct SolveArgs {
  DEarly E;
  const uint16_t* ids;
  const float* pos;
  uint32_t n_src;
  const omg_chain* chains;
  uint32_t n_chains;
  float lx, ly, lz;
  const omg_aabb* extras;
  uint32_t n_extras;
  omg_mesh_record* out;
};

__global__ void __launch_bounds__(128) early_solve_kernel(SolveArgs A) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (uint64_t)A.n_src * A.n_chains) return;
  const uint32_t s = (uint32_t)(k / A.n_chains), c = (uint32_t)(k % A.n_chains);
  SegList L;
  omg_mesh_record r;
  const omg_chain ch = A.chains[c];
  if (!mesh_record(A.E, ch, A.ids[s], A.pos[3 * s], A.pos[3 * s + 1], A.pos[3 * s + 2], A.lx, A.ly, A.lz, A.extras,
                   A.n_extras, L, r)) {
    r.source = A.ids[s];
    for (int q = 0; q < OMG_CHAIN_MAX_ORDER; q++) r.chain[q] = ch.surf[q];
    r.order = ch.order;
    r.delay_s = 0.0f;
    r.dir[0] = r.dir[1] = r.dir[2] = 0.0f;
    r.gains[0] = r.gains[1] = r.gains[2] = 0.0f;
    r.key = 0u;
    r.valid = 0u;
  }
  A.out[k] = r;
}

}  // namespace

cudaError_t launch_early_discover(const DEarly& E, const float lis[3], uint32_t n_rays, uint32_t rot, bool use_boxes,
                                  const float* jitter, unsigned long long* cand_key, omg_chain* cand_chain,
                                  uint32_t* cand_slot, unsigned long long* tkey, uint32_t* tidx, uint32_t tcap,
                                  omg_chain* out, uint32_t cap, uint32_t* n_out, cudaStream_t s) {
  DiscArgs A;
  A.E = E;
  A.lx = lis[0];
  A.ly = lis[1];
  A.lz = lis[2];
  A.n_rays = n_rays;
  A.rot = rot;
  A.use_boxes = use_boxes ? 1u : 0u;
  A.ga = 3.14159265358979323846f * (3.0f - sqrtf(5.0f));
  A.jitter = jitter;
  A.cand_key = cand_key;
  A.cand_chain = cand_chain;
  A.cand_slot = cand_slot;
  A.tkey = tkey;
  A.tidx = tidx;
  A.tcap = tcap;
  if (n_rays) early_discover_kernel<<<(n_rays + 127) / 128, 128, 0, s>>>(A);
  early_compact_kernel<<<1, kCompactThreads, 0, s>>>(cand_key, cand_chain, cand_slot, tidx, 3u * n_rays, out, cap,
                                                     n_out);
  return cudaGetLastError();
}

cudaError_t launch_early_solve(const DEarly& E, const uint16_t* ids, const float* pos, uint32_t n_src,
                               const omg_chain* chains, uint32_t n_chains, const float lis[3], const omg_aabb* extras,
                               uint32_t n_extras, omg_mesh_record* out, cudaStream_t s) {
  SolveArgs A;
  A.E = E;
  A.ids = ids;
  A.pos = pos;
  A.n_src = n_src;
  A.chains = chains;
  A.n_chains = n_chains;
  A.lx = lis[0];
  A.ly = lis[1];
  A.lz = lis[2];
  A.extras = extras;
  A.n_extras = n_extras;
  A.out = out;
  const uint64_t n = (uint64_t)n_src * n_chains;
  if (n == 0) return cudaSuccess;
  early_solve_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(A);
  return cudaGetLastError();
}

}  // namespace omg
