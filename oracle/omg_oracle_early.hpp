// CPU oracle for the world-mesh early reflections — TEST INFRASTRUCTURE.
//
// Restates crates/omg-core/src/pt_mesh.rs (surface chains over the world
// mesh: the surface table, chain discovery from the listener, and the exact
// per-chain solve with transmission along every leg), with Aabb::clip from
// crates/omg-core/src/pt.rs:43-70 and reflection_amplitude / air_attenuation
// from crates/omg-core/src/material.rs:65-84. f32 arithmetic in the
// reference's operation order (compiled with -ffp-contract=off); the only
// transcendentals (cos/sin of the fan azimuth, exp of the air attenuation)
// are evaluated in double and rounded once, as the CUDA library does.
//
// Only the test suite and the benchmark's CPU leg load this code.
#pragma once
#include <set>

#include "omg_oracle.hpp"

namespace orc {

constexpr int M_MAX_ORDER = 3;           // pt_mesh.rs:23
constexpr float MIN_DIST = 0.3f;         // pt_mesh.rs:24
constexpr uint16_t NO_SURF = 0xFFFF;     // pt_mesh.rs:25
constexpr float AUDIBLE_FLOOR = 2e-5f;   // pt_mesh.rs:27
constexpr float SPEED_OF_SOUND = 343.0f; // lib.rs:18
constexpr float AIR_ABSORPTION_PER_M[3] = {1.0e-4f, 5.0e-4f, 3.0e-3f};  // material.rs:76

// pt.rs:31-35
struct Aabb {
  float mn[3], mx[3];
  float transmission[3];
};

// pt.rs:43-70: the interior crossing of a->b, or none.
inline bool aabb_clip(const Aabb& x, const V3<float>& a, const V3<float>& b) {
  const V3<float> d = b - a;
  float t0 = 0.0f, t1 = 1.0f;
  for (int axis = 0; axis < 3; axis++) {
    const float da = d.get(axis), aa = a.get(axis), mn = x.mn[axis], mx = x.mx[axis];
    if (std::fabs(da) < 1e-9f) {
      if (aa < mn || aa > mx) return false;
    } else {
      float ta = (mn - aa) / da, tb = (mx - aa) / da;
      if (ta > tb) std::swap(ta, tb);
      t0 = std::fmax(t0, ta);
      t1 = std::fmin(t1, tb);
      if (t0 > t1) return false;
    }
  }
  return t1 > 1e-4f && t0 < 1.0f - 1e-4f;
}

// material.rs:78-84 (exp in double, rounded once)
inline void air_attenuation(float dist, float out[3]) {
  for (int b = 0; b < 3; b++) out[b] = (float)std::exp((double)(-AIR_ABSORPTION_PER_M[b] * dist));
}

// pt_mesh.rs:30-41
struct Surface {
  V3<float> n;
  float d;
  float refl[3], trans[3];
  bool rect;
  V3<float> fmin, fmax;
};

// pt_mesh.rs:44-110
struct SurfaceTable {
  std::vector<Surface> surfaces;
  uint16_t base_overlay = 0;

  static void material_amps(const Material& m, float refl[3], float trans[3]) {
    for (int b = 0; b < 3; b++) {
      refl[b] = std::sqrt(std::fmax(1.0f - m.absorption[b], 0.0f));  // material.rs:65-71
      trans[b] = m.transmission[b];
    }
  }

  void build(const Mesh<float>& mesh) {  // pt_mesh.rs:51-78
    surfaces.clear();
    std::vector<bool> set;
    for (uint32_t t = 0; t < (uint32_t)mesh.tri_count(); t++) {
      const size_t sid = mesh.tri_surface[t];
      if (sid >= surfaces.size()) {
        Surface blank{};
        blank.n = V3<float>(0, 0, 1);
        blank.d = std::numeric_limits<float>::max();
        surfaces.resize(sid + 1, blank);
        set.resize(sid + 1, false);
      }
      if (!set[sid]) {
        Surface& s = surfaces[sid];
        s.n = mesh.tri_normal(t);
        s.d = s.n.dot(mesh.positions[mesh.indices[3 * t]]);
        material_amps(mesh.materials[mesh.tri_material[t]], s.refl, s.trans);
        s.rect = false;
        set[sid] = true;
      }
    }
    base_overlay = (uint16_t)surfaces.size();
  }

  void append_box(const float mn[3], const float mx[3], const Material& m) {  // pt_mesh.rs:86-109
    for (int axis = 0; axis < 3; axis++) {
      for (int side = 0; side < 2; side++) {
        Surface s{};
        s.n = V3<float>(0, 0, 0);
        s.n.set(axis, side == 0 ? -1.0f : 1.0f);
        const float plane = side == 0 ? mn[axis] : mx[axis];
        s.fmin = V3<float>(mn[0], mn[1], mn[2]);
        s.fmax = V3<float>(mx[0], mx[1], mx[2]);
        s.fmin.set(axis, plane);
        s.fmax.set(axis, plane);
        s.d = s.n.dot(side == 0 ? V3<float>(mn[0], mn[1], mn[2]) : V3<float>(mx[0], mx[1], mx[2]));
        material_amps(m, s.refl, s.trans);
        s.rect = true;
        surfaces.push_back(s);
      }
    }
  }
};

struct MChain {
  uint16_t c[M_MAX_ORDER];
  uint8_t order;
};

// pt_mesh.rs:113-121
struct MeshRecord {
  uint16_t source;
  uint16_t chain[M_MAX_ORDER];
  uint8_t order;
  float delay_s;
  float dir[3];
  float gains[3];
};

// pt_mesh.rs:123-134 (FNV-1a over source and surface ids)
inline uint32_t record_key(const MeshRecord& r) {
  uint32_t h = 0x811C9DC5u ^ (uint32_t)r.source;
  for (int i = 0; i < r.order; i++) h = (h ^ (uint32_t)r.chain[i]) * 16777619u;
  return (h ^ 0xA5u) * 16777619u;
}

// pt_mesh.rs:136-138
inline V3<float> mirror(const V3<float>& p, const Surface& s) {
  return p - s.n * (2.0f * (s.n.dot(p) - s.d));
}

// pt_mesh.rs:146-182
inline bool leg_transmission(const Mesh<float>& mesh, const V3<float>& a, const V3<float>& b, bool has_skip,
                             uint16_t skip_sid, float t_expect, const std::vector<Aabb>& extras,
                             std::vector<SegHit>& buf, float trans[3]) {
  mesh.segment_hits(a, b, buf);
  const float seg_len = std::fmax((b - a).length(), 1e-6f);
  auto dead = [&]() { return trans[0] < 1e-6f && trans[1] < 1e-6f && trans[2] < 1e-6f; };
  for (const SegHit& h : buf) {
    if (has_skip && mesh.tri_surface[h.tri] == skip_sid && std::fabs((float)h.t - t_expect) * seg_len < 0.05f)
      continue;
    const Material& m = mesh.materials[h.material];
    for (int k = 0; k < 3; k++) trans[k] *= m.transmission[k];
    if (dead()) return false;
  }
  for (const Aabb& x : extras) {
    if (aabb_clip(x, a, b)) {
      for (int k = 0; k < 3; k++) trans[k] *= x.transmission[k];
      if (dead()) return false;
    }
  }
  return true;
}

inline bool all_below(const float v[3], float lim) { return v[0] < lim && v[1] < lim && v[2] < lim; }

// pt_mesh.rs:186-337
inline bool mesh_record(const Mesh<float>& mesh, const SurfaceTable& table, const uint16_t* chain, int order,
                        uint16_t source, const V3<float>& src, const V3<float>& listener,
                        const std::vector<Aabb>& extras, std::vector<SegHit>& buf, MeshRecord* out) {
  V3<float> img = src;
  for (int i = order - 1; i >= 0; i--) {
    if (chain[i] >= table.surfaces.size()) return false;
    img = mirror(img, table.surfaces[chain[i]]);
  }
  const V3<float> to_img = img - listener;
  const float dist = to_img.length();
  if (dist < 1e-4f) return false;
  const V3<float> dir = to_img * (1.0f / dist);

  float gm[3] = {1.0f, 1.0f, 1.0f};
  V3<float> pos = listener, d = dir;
  for (int i = 0; i < order; i++) {
    const uint16_t sid = chain[i];
    if (sid >= table.surfaces.size()) return false;
    const Surface& s = table.surfaces[sid];
    const float denom = s.n.dot(d);
    if (std::fabs(denom) < 1e-9f) return false;
    const float t = (s.d - s.n.dot(pos)) / denom;
    if (t <= 1e-4f) return false;
    const V3<float> hit = pos + d * t;
    float rt;
    uint32_t rtri;
    if (s.rect) {
      const float eps = 1e-3f;
      for (int a = 0; a < 3; a++)
        if (hit.get(a) < s.fmin.get(a) - eps || hit.get(a) > s.fmax.get(a) + eps) return false;
      if (mesh.raycast(pos + d * 1e-4f, d, &rt, &rtri) && rt < t - 1e-3f) {
        const Material& m = mesh.materials[mesh.tri_material[rtri]];
        if (all_below(m.transmission, 1e-6f)) return false;
      }
    } else {
      if (!mesh.raycast(pos + d * 1e-4f, d, &rt, &rtri)) return false;
      const bool on_surface = mesh.tri_surface[rtri] == sid && std::fabs(rt - t) < 2e-2f;
      if (!on_surface) {
        if (rt < t - 1e-3f) {
          const Material& m = mesh.materials[mesh.tri_material[rtri]];
          if (all_below(m.transmission, 1e-4f)) return false;
          mesh.segment_hits(pos, hit + d * 0.05f, buf);
          bool found = false;
          for (const SegHit& h : buf)
            if (mesh.tri_surface[h.tri] == sid && std::fabs((float)h.t * (t + 0.05f) - t) < 0.1f) found = true;
          if (!found) return false;
        } else {
          return false;
        }
      }
    }
    if (!leg_transmission(mesh, pos, hit, true, sid, 1.0f, extras, buf, gm)) return false;
    for (int k = 0; k < 3; k++) gm[k] *= s.refl[k];
    pos = hit + s.n * (s.n.dot(d) < 0.0f ? 1e-4f : -1e-4f);
    d = d - s.n * (2.0f * s.n.dot(d));
  }
  if (order > 0) {
    const Surface& s = table.surfaces[chain[order - 1]];
    if ((s.n.dot(pos) - s.d) * (s.n.dot(src) - s.d) < 0.0f) return false;
  }
  if (!leg_transmission(mesh, pos, src, false, 0, 0.0f, extras, buf, gm)) return false;
  if (order > 0) {
    const V3<float> to_src = src - pos;
    const float leg = to_src.length();
    if (leg > 1e-4f && (to_src * (1.0f / leg)).dot(d) < 0.995f) return false;
  }
  const float dtot = std::fmax(dist, MIN_DIST);
  float air[3];
  air_attenuation(dtot, air);
  float gains[3];
  for (int k = 0; k < 3; k++) gains[k] = air[k] / dtot * gm[k];
  if (all_below(gains, AUDIBLE_FLOOR)) return false;
  out->source = source;
  for (int i = 0; i < M_MAX_ORDER; i++) out->chain[i] = i < order ? chain[i] : NO_SURF;
  out->order = (uint8_t)order;
  out->delay_s = dist / SPEED_OF_SOUND;
  out->dir[0] = dir.x;
  out->dir[1] = dir.y;
  out->dir[2] = dir.z;
  for (int k = 0; k < 3; k++) out->gains[k] = gains[k];
  return true;
}

// pt_mesh.rs:382-457: listener-launched rotating golden fan, specular
// bounces, chains of surface ids in first-found order.
inline void mesh_chains(const Mesh<float>& mesh, const std::vector<std::pair<V3<float>, V3<float>>>& boxes,
                        uint16_t base, const V3<float>& listener, uint32_t n_rays, uint32_t rot,
                        std::vector<MChain>& out) {
  std::set<uint64_t> seen;
  const float ga = 3.14159265358979323846f * (3.0f - std::sqrt(5.0f));
  Xorshift64 jitter((0xC6Bull ^ (uint64_t)rot) | 1ull);
  const float tau = 6.28318530717958647692f;
  for (uint32_t i = 0; i < n_rays; i++) {
    const float z = 1.0f - 2.0f * ((float)i + 0.5f) / (float)n_rays;
    const float r = std::sqrt(std::fmax(1.0f - z * z, 0.0f));
    const float phi = ga * (float)i + (float)rot * 0.61803398875f * tau + jitter.next_f32() * 0.02f;
    float sp, cp;
    sincos_r(phi, &sp, &cp);
    V3<float> dir(r * cp, r * sp, z);
    V3<float> pos = listener;
    MChain chain;
    for (int k = 0; k < M_MAX_ORDER; k++) chain.c[k] = NO_SURF;
    for (int k = 0; k < M_MAX_ORDER; k++) {
      float mt;
      uint32_t mtri;
      const bool mh = mesh.raycast(pos, dir, &mt, &mtri);
      float t = mh ? mt : std::numeric_limits<float>::max();
      bool has_sid = mh;
      uint16_t sid = mh ? mesh.tri_surface[mtri] : 0;
      V3<float> normal = mh ? mesh.tri_normal(mtri) : V3<float>(0, 0, 1);
      for (size_t bi = 0; bi < boxes.size(); bi++) {
        const V3<float>& mn = boxes[bi].first;
        const V3<float>& mx = boxes[bi].second;
        float t0 = 1e-4f, t1 = t;
        int axis = 3;
        for (int a = 0; a < 3; a++) {
          const float da = dir.get(a);
          if (std::fabs(da) < 1e-9f) {
            if (pos.get(a) < mn.get(a) || pos.get(a) > mx.get(a)) {
              t0 = std::numeric_limits<float>::max();
              break;
            }
          } else {
            float ta = (mn.get(a) - pos.get(a)) / da, tb = (mx.get(a) - pos.get(a)) / da;
            if (ta > tb) std::swap(ta, tb);
            if (ta > t0) {
              t0 = ta;
              axis = a;
            }
            t1 = std::fmin(t1, tb);
            if (t0 > t1) {
              t0 = std::numeric_limits<float>::max();
              break;
            }
          }
        }
        if (t0 < t && axis < 3) {
          t = t0;
          const int face = axis * 2 + (dir.get(axis) > 0.0f ? 0 : 1);
          has_sid = true;
          sid = (uint16_t)(base + (uint16_t)(bi * 6 + face));
          V3<float> n(0, 0, 0);
          n.set(axis, dir.get(axis) > 0.0f ? -1.0f : 1.0f);
          normal = n;
        }
      }
      if (!has_sid) break;
      if (t <= 1e-4f || t > 200.0f) break;
      pos = pos + dir * t;
      chain.c[k] = sid;
      uint64_t key = 1;
      for (int q = 0; q <= k; q++) key = key * 65536ull + (uint64_t)chain.c[q] + 1ull;
      if (seen.insert(key).second) {
        MChain c = chain;
        c.order = (uint8_t)(k + 1);
        out.push_back(c);
      }
      const V3<float> n = normal.dot(dir) > 0.0f ? normal * -1.0f : normal;
      dir = dir - n * (2.0f * dir.dot(n));
      pos = pos + n * 1e-4f;
    }
  }
}

}  // namespace orc
