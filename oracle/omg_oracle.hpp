// CPU oracle for the stochastic energy path tracer — TEST INFRASTRUCTURE.
//
// This file restates omg-audio's CPU tracer (crates/omg-core) and ambient dome
// (crates/omg-scene/src/dome.rs) so the CUDA library can be checked against
// it. It is templated on the real type R:
//   R = float  : the reference's own f32 semantics (operation order kept,
//                compiled with -ffp-contract=off so nothing is fused);
//   R = double : the FP64 oracle the GPU results are judged against.
// Material constants, positions and poses are f32 inputs in the reference;
// the FP64 oracle promotes them exactly.
//
// Only the test suite, the smoke check and the benchmark's CPU-baseline leg
// may load this code. Nothing in the product links it.
//
// Every function cites the reference file:line it follows.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <unordered_map>
#include <vector>

namespace orc {

constexpr int MAXB = 8;           // band capacity of the runtime band count
constexpr uint32_t LEAF_BIT = 1u << 31;   // mesh.rs:17
constexpr int LEAF_SIZE = 4;              // mesh.rs:16
constexpr float MAX_PRIM_EDGE = 4.0f;     // mesh.rs:41

// ----------------------------------------------------------------- vec3
// crates/omg-core/src/vec3.rs:1-82
template <class R>
struct V3 {
  R x, y, z;
  V3() : x(0), y(0), z(0) {}
  V3(R a, R b, R c) : x(a), y(b), z(c) {}
  R dot(const V3& o) const { return x * o.x + y * o.y + z * o.z; }
  R length() const { return std::sqrt(dot(*this)); }
  V3 operator+(const V3& o) const { return V3(x + o.x, y + o.y, z + o.z); }
  V3 operator-(const V3& o) const { return V3(x - o.x, y - o.y, z - o.z); }
  V3 operator*(R s) const { return V3(x * s, y * s, z * s); }
  V3 cross(const V3& o) const {
    return V3(y * o.z - z * o.y, z * o.x - x * o.z, x * o.y - y * o.x);
  }
  // vec3.rs:19-26: multiply by the reciprocal, (1,0,0) for tiny vectors
  V3 normalize() const {
    R l = length();
    if (l > R(1e-12)) return (*this) * (R(1) / l);
    return V3(1, 0, 0);
  }
  // Rust f32::min/max return the non-NaN operand, as fmin/fmax do.
  V3 vmin(const V3& o) const { return V3(std::fmin(x, o.x), std::fmin(y, o.y), std::fmin(z, o.z)); }
  V3 vmax(const V3& o) const { return V3(std::fmax(x, o.x), std::fmax(y, o.y), std::fmax(z, o.z)); }
  R get(int a) const { return a == 0 ? x : (a == 1 ? y : z); }
  void set(int a, R v) { if (a == 0) x = v; else if (a == 1) y = v; else z = v; }
};

template <class R>
inline V3<R> from_f(const float* p) { return V3<R>(R(p[0]), R(p[1]), R(p[2])); }

// f32 -> usize as Rust's `as` does it: saturating, NaN -> 0.
template <class R>
inline uint64_t sat_u64(R v) {
  if (!(v >= R(0))) return 0;
  if (v >= R(1.8446744073709552e19)) return UINT64_MAX;
  return (uint64_t)v;
}

// cos/sin of an f32 angle, correctly rounded to R: evaluated in double and
// rounded once (the CUDA library does the same, so both sides agree bit for
// bit on every direction a ray ever takes).
template <class R>
inline void sincos_r(R phi, R* s, R* c) {
  double dphi = (double)phi;
  *s = (R)std::sin(dphi);
  *c = (R)std::cos(dphi);
}

// ----------------------------------------------------------------- material
// crates/omg-core/src/material.rs:7-16 (absorption/scattering/transmission
// per band); band count is a runtime value here (3 in the reference).
struct Material {
  float absorption[MAXB];
  float scattering;
  float transmission[MAXB];
};

// ----------------------------------------------------------------- RNGs
// crates/omg-core/src/rng.rs:2-30 — xorshift64*, the reference CPU stream
// (one sequential stream shared by every ray of a trace, tracer.rs:86,94).
struct Xorshift64 {
  uint64_t s;
  explicit Xorshift64(uint64_t seed) : s(seed < 1 ? 1 : seed) {}      // rng.rs:5-7
  uint64_t next_u64() {                                                // rng.rs:9-16
    uint64_t x = s;
    x ^= x >> 12;
    x ^= x << 25;
    x ^= x >> 27;
    s = x;
    return x * 0x2545F4914F6CDD1DULL;
  }
  float next_f32() { return (float)(next_u64() >> 40) / (float)(1ULL << 24); }  // rng.rs:19-21
};

// crates/omg-gpu/shaders/trace_mesh.wgsl:90-98, 211-213 — the per-ray
// counter-based PCG-RXS-M-XS stream: state = (seed ^ ray*0x9E3779B9) + 1,
// two warm-up draws. The CUDA kernels use exactly this stream.
struct PcgRay {
  uint32_t s;
  PcgRay(uint32_t seed, uint32_t ray) {
    s = (seed ^ (ray * 0x9E3779B9u)) + 1u;
    next_u32();
    next_u32();
  }
  uint32_t next_u32() {
    s = s * 747796405u + 2891336453u;
    uint32_t word = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (word >> 22u) ^ word;
  }
  float next_f32() { return (float)(next_u32() >> 8u) / 16777216.0f; }
};

// sin and cos of an angle in [0, 2*pi] in f32 only, the same operations in the
// same order as the CUDA kernel's: Cody-Waite reduction by pi/2 (three-part
// constant, exact quadrant products) and Taylor polynomials on [-pi/4, pi/4]
// with coefficients +-1/n!. Within 3 ulp of the true values.
inline void sincos_f32(float phi, float* s, float* c) {
  const float k = std::nearbyint(phi * 0.636619772367581343f);
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
  if (q == 0) { *s = sp; *c = cp; }
  else if (q == 1) { *s = cp; *c = -sp; }
  else if (q == 2) { *s = -sp; *c = -cp; }
  else { *s = -cp; *c = sp; }
}

// the ray directions' sin/cos: f32 polynomial (as the GPU), exact in FP64
inline void dir_sincos(float phi, float* s, float* c) { sincos_f32(phi, s, c); }
inline void dir_sincos(double phi, double* s, double* c) { *s = std::sin(phi); *c = std::cos(phi); }

// rng.rs:24-29 — z = 1-2u, phi = TAU*u. The draws are f32 in the reference;
// the FP64 oracle takes the same f32 draws and continues in R.
template <class R, class G>
inline V3<R> unit_sphere(G& g) {
  const float TAU = 6.28318530717958647692f;
  float u1 = g.next_f32();
  R z = R(1) - R(2) * R(u1);
  R r = std::sqrt(std::fmax(R(1) - z * z, R(0)));
  float u2 = g.next_f32();
  R phi = R(TAU) * R(u2);
  R s, c;
  dir_sincos(phi, &s, &c);
  return V3<R>(r * c, r * s, z);
}

// ----------------------------------------------------------------- geometry
// Traversal counters. The reference's ordered walk (mesh.rs:484-541) reads a
// popped node's record, and for an internal node both children's records (their
// boxes); a child popped later is the record its parent already read. So the
// DISTINCT 32-byte records a closest-hit query touches are the root plus the
// children of every internal node it processes: unique_nodes = queries +
// child_boxes. node_reads counts every read, repeats included.
struct TraversalStats {
  uint64_t node_reads = 0;       // BvhNode records read, repeats included (32 B each in the flattened layout)
  uint64_t prim_tests = 0;       // PackedTri records tested (48 B each)
  uint64_t queries = 0;          // closest-hit or crossing queries
  uint64_t internal_visits = 0;  // internal nodes popped and processed
  uint64_t leaf_visits = 0;      // leaves popped and processed
  uint64_t child_boxes = 0;      // child boxes read by internal visits (2 each)
  uint64_t unique_nodes = 0;     // distinct node records touched per query, summed over queries
};

template <class R>
struct GeomHit {        // scene.rs:5-10
  R t;
  V3<R> normal;         // oriented against the incoming ray
  const Material* material;
};

// scene.rs:27-88 — analytic shoebox [0,size]^3, wall order x-,x+,y-,y+,z-,z+.
template <class R>
struct Shoebox {
  V3<R> size;
  Material walls[6];
  bool contains(const V3<R>& p) const {   // scene.rs:39-41
    return p.x > 0 && p.x < size.x && p.y > 0 && p.y < size.y && p.z > 0 && p.z < size.z;
  }
  void raycast(const V3<R>& p, const V3<R>& d, R* best_t, int* best_w) const {  // scene.rs:45-62
    R bt = R(std::numeric_limits<float>::max());
    int bw = 0;
    for (int axis = 0; axis < 3; axis++) {
      R di = d.get(axis);
      if (di > R(1e-9)) {
        R t = (size.get(axis) - p.get(axis)) / di;
        if (t < bt) { bt = t; bw = 2 * axis + 1; }
      } else if (di < R(-1e-9)) {
        R t = -p.get(axis) / di;
        if (t < bt) { bt = t; bw = 2 * axis; }
      }
    }
    *best_t = bt;
    *best_w = bw;
  }
  bool raycast_hit(const V3<R>& p, const V3<R>& d, GeomHit<R>* h, TraversalStats* = nullptr,
                   uint32_t* = nullptr) const {  // scene.rs:64-88
    if (!contains(p)) return false;
    R t; int wall;
    raycast(p, d, &t, &wall);
    if (!std::isfinite(t) || t <= R(0)) return false;
    V3<R> n(0, 0, 0);
    n.set(wall / 2, (wall % 2 == 0) ? R(1) : R(-1));
    h->t = t;
    h->normal = n;
    h->material = &walls[wall];
    return true;
  }
};

// scene.rs:90-137 — axis-aligned panel overlay (door leaves, panes).
template <class R>
struct BoxPanel {
  V3<R> mn, mx;
  Material m;
};

// ----------------------------------------------------------------- mesh
struct PackedTriF { float a[3], e1[3], e2[3]; uint32_t tri; uint16_t material; };

template <class R>
struct PackedTri {      // mesh.rs:43-50
  V3<R> a, e1, e2;
  uint32_t tri;
  uint16_t material;
};

template <class R>
struct BvhNode {        // mesh.rs:52-58
  V3<R> bmin, bmax;
  uint32_t a, b;
};

struct SegHit { double t; uint32_t tri; uint16_t material; };  // mesh.rs:61-68


// mesh.rs:70-165 — incremental assembly with 0.1 mm vertex dedup.
struct MeshBuilder {
  std::vector<float> positions;          // xyz triples (f32, as the reference)
  std::vector<uint32_t> indices;         // 3 per tri
  std::vector<uint16_t> tri_material;
  std::vector<Material> materials;
  std::vector<uint16_t> tri_surface;
  std::vector<float> tri_max_edge;
  float cur_max_edge = 0.0f;
  uint16_t next_surface = 0;
  struct KeyHash {
    size_t operator()(const std::tuple<int64_t, int64_t, int64_t>& k) const {
      uint64_t h = (uint64_t)std::get<0>(k) * 0x9E3779B97F4A7C15ULL;
      h ^= (uint64_t)std::get<1>(k) + 0x7F4A7C159E3779B9ULL + (h << 6) + (h >> 2);
      h ^= (uint64_t)std::get<2>(k) + 0x94D049BB133111EBULL + (h << 6) + (h >> 2);
      return (size_t)h;
    }
  };
  std::unordered_map<std::tuple<int64_t, int64_t, int64_t>, uint32_t, KeyHash> lookup;

  uint16_t material(const Material& m) {            // mesh.rs:93-96
    materials.push_back(m);
    return (uint16_t)(materials.size() - 1);
  }
  uint16_t begin_surface() { next_surface++; return (uint16_t)(next_surface - 1); }  // mesh.rs:103-106
  void coarse(float e) { cur_max_edge = e; }        // mesh.rs:132-134
  // mesh.rs:108-114: key = round(v * 1e4) in f32, ties away from zero
  uint32_t vertex(const float p[3]) {
    auto q = [](float v) { return (int64_t)std::round(v * 1e4f); };
    auto key = std::make_tuple(q(p[0]), q(p[1]), q(p[2]));
    auto it = lookup.find(key);
    if (it != lookup.end()) return it->second;
    positions.push_back(p[0]); positions.push_back(p[1]); positions.push_back(p[2]);
    uint32_t id = (uint32_t)(positions.size() / 3 - 1);
    lookup.emplace(key, id);
    return id;
  }
  void tri(const float a[3], const float b[3], const float c[3], uint16_t m) {  // mesh.rs:116-126
    uint32_t ia = vertex(a), ib = vertex(b), ic = vertex(c);
    indices.push_back(ia); indices.push_back(ib); indices.push_back(ic);
    tri_material.push_back(m);
    tri_surface.push_back(next_surface > 0 ? (uint16_t)(next_surface - 1) : 0);
    tri_max_edge.push_back(cur_max_edge > 0.0f ? cur_max_edge : MAX_PRIM_EDGE);
  }
  void quad(const float a[3], const float b[3], const float c[3], const float d[3], uint16_t m) {  // mesh.rs:137-140
    tri(a, b, c, m);
    tri(a, c, d, m);
  }
  void abox(const float mn[3], const float mx[3], uint16_t m) {  // mesh.rs:144-153
    float ax = mn[0], ay = mn[1], az = mn[2], bx = mx[0], by = mx[1], bz = mx[2];
    auto Q = [&](float p0, float p1, float p2, float q0, float q1, float q2, float r0, float r1, float r2,
                 float s0, float s1, float s2) {
      float A[3] = {p0, p1, p2}, B[3] = {q0, q1, q2}, C[3] = {r0, r1, r2}, D[3] = {s0, s1, s2};
      quad(A, B, C, D, m);
    };
    Q(ax, ay, az, ax, by, az, ax, by, bz, ax, ay, bz);
    Q(bx, ay, az, bx, ay, bz, bx, by, bz, bx, by, az);
    Q(ax, ay, az, ax, ay, bz, bx, ay, bz, bx, ay, az);
    Q(ax, by, az, bx, by, az, bx, by, bz, ax, by, bz);
    Q(ax, ay, az, bx, ay, az, bx, by, az, ax, by, az);
    Q(ax, ay, bz, ax, by, bz, bx, by, bz, bx, ay, bz);
  }
};

template <class R>
struct Mesh {
  std::vector<V3<R>> positions;
  std::vector<uint32_t> indices;
  std::vector<uint16_t> tri_material;
  std::vector<Material> materials;
  std::vector<uint16_t> tri_surface;
  std::vector<float> tri_max_edge;
  std::vector<BvhNode<R>> nodes;
  std::vector<PackedTri<R>> packed;

  size_t tri_count() const { return tri_material.size(); }
  void tri_verts(uint32_t t, V3<R>* a, V3<R>* b, V3<R>* c) const {
    *a = positions[indices[3 * t + 0]];
    *b = positions[indices[3 * t + 1]];
    *c = positions[indices[3 * t + 2]];
  }
  V3<R> tri_normal(uint32_t t) const {  // mesh.rs:458-461
    V3<R> a, b, c;
    tri_verts(t, &a, &b, &c);
    return (b - a).cross(c - a).normalize();
  }

  // mesh.rs:241-287 — tessellate oversized tris (midpoint of the longest
  // edge, LIFO work list), then the binned-SAH build.
  void build_bvh() {
    nodes.clear();
    std::vector<PackedTri<R>> prims;
    prims.reserve(tri_count());
    struct W { V3<R> a, b, c; uint32_t t; };
    std::vector<W> work;
    work.reserve(tri_count());
    for (uint32_t t = 0; t < (uint32_t)tri_count(); t++) {
      W w; tri_verts(t, &w.a, &w.b, &w.c); w.t = t;
      work.push_back(w);
    }
    while (!work.empty()) {
      W w = work.back();
      work.pop_back();
      V3<R> a = w.a, b = w.b, c = w.c;
      uint32_t t = w.t;
      R lab = (b - a).length(), lbc = (c - b).length(), lca = (a - c).length();
      R longest = std::fmax(std::fmax(lab, lbc), lca);
      if (longest > R(tri_max_edge[t])) {
        if (lab >= lbc && lab >= lca) {
          V3<R> m = (a + b) * R(0.5);
          work.push_back({a, m, c, t});
          work.push_back({m, b, c, t});
        } else if (lbc >= lca) {
          V3<R> m = (b + c) * R(0.5);
          work.push_back({a, b, m, t});
          work.push_back({a, m, c, t});
        } else {
          V3<R> m = (c + a) * R(0.5);
          work.push_back({a, b, m, t});
          work.push_back({m, b, c, t});
        }
        continue;
      }
      PackedTri<R> p;
      p.a = a; p.e1 = b - a; p.e2 = c - a; p.tri = t; p.material = tri_material[t];
      prims.push_back(p);
    }
    if (prims.empty()) { packed.swap(prims); return; }
    size_t n = prims.size();
    build_node(prims, 0, n);
    packed.swap(prims);
    // near-tie walks test boxes grown by 2^-19 M_a + 2^-17 x the longest
    // primitive edge (M_a: the largest |box coordinate| on axis a plus 1 m), so
    // that they find every hit Möller–Trumbore accepts, even just outside a
    // triangle's bounds; the CUDA walks grow theirs the same way
    double mx[3] = {0, 0, 0}, e = 0;
    for (const BvhNode<R>& nd : nodes)
      for (int a = 0; a < 3; a++)
        mx[a] = std::max(mx[a], std::max(std::fabs((double)nd.bmin.get(a)), std::fabs((double)nd.bmax.get(a))));
    for (const PackedTri<R>& p : packed) {
      const V3<R> e3 = p.e2 - p.e1;
      e = std::max(e, std::max((double)p.e1.length(), std::max((double)p.e2.length(), (double)e3.length())));
    }
    for (int a = 0; a < 3; a++) tie_grow[a] = R(std::ldexp(mx[a] + 1.0, -19) + std::ldexp(e, -17));
  }
  R tie_grow[3] = {0, 0, 0};

  // mesh.rs:292-405 — 16-bin SAH on the widest centroid axis, leaf <= 4,
  // median fallback, stable two-pointer partition.
  uint32_t build_node(std::vector<PackedTri<R>>& prims, size_t start, size_t end) {
    const int NBIN = 16;
    const R FMAX = R(std::numeric_limits<float>::max());
    const R FMIN = R(-std::numeric_limits<float>::max());
    auto pbounds = [](const PackedTri<R>& p, V3<R>* lo, V3<R>* hi) {
      V3<R> a = p.a, b = p.a + p.e1, c = p.a + p.e2;
      *lo = a.vmin(b).vmin(c);
      *hi = a.vmax(b).vmax(c);
    };
    auto pcentroid = [](const PackedTri<R>& p) { return p.a + (p.e1 + p.e2) * (R(1) / R(3)); };
    auto area = [](const V3<R>& lo, const V3<R>& hi) {
      V3<R> e = (hi - lo).vmax(V3<R>(0, 0, 0));
      return R(2) * (e.x * e.y + e.y * e.z + e.z * e.x);
    };
    V3<R> bmin(FMAX, FMAX, FMAX), bmax(FMIN, FMIN, FMIN), cmin = bmin, cmax = bmax;
    for (size_t i = start; i < end; i++) {
      V3<R> lo, hi;
      pbounds(prims[i], &lo, &hi);
      bmin = bmin.vmin(lo);
      bmax = bmax.vmax(hi);
      V3<R> c = pcentroid(prims[i]);
      cmin = cmin.vmin(c);
      cmax = cmax.vmax(c);
    }
    uint32_t idx = (uint32_t)nodes.size();
    nodes.push_back({bmin, bmax, 0, 0});
    size_t count = end - start;
    if (count <= (size_t)LEAF_SIZE) {
      nodes[idx].a = LEAF_BIT | (uint32_t)start;
      nodes[idx].b = (uint32_t)count;
      return idx;
    }
    V3<R> cext = cmax - cmin;
    int axis = (cext.x >= cext.y && cext.x >= cext.z) ? 0 : (cext.y >= cext.z ? 1 : 2);
    R cwidth = cext.get(axis);
    size_t mid;
    if (cwidth < R(1e-6)) {
      mid = start + count / 2;
    } else {
      auto bin_of = [&](const PackedTri<R>& p) -> int {
        R v = (pcentroid(p).get(axis) - cmin.get(axis)) / cwidth * R(NBIN);
        v = std::fmin(v, R(NBIN) - R(1));
        return (int)sat_u64<R>(v);
      };
      V3<R> bnlo[NBIN], bnhi[NBIN];
      uint32_t bnn[NBIN];
      for (int k = 0; k < NBIN; k++) { bnlo[k] = V3<R>(FMAX, FMAX, FMAX); bnhi[k] = V3<R>(FMIN, FMIN, FMIN); bnn[k] = 0; }
      for (size_t i = start; i < end; i++) {
        int k = bin_of(prims[i]);
        V3<R> lo, hi;
        pbounds(prims[i], &lo, &hi);
        bnlo[k] = bnlo[k].vmin(lo);
        bnhi[k] = bnhi[k].vmax(hi);
        bnn[k] += 1;
      }
      R right_cost[NBIN];
      for (int k = 0; k < NBIN; k++) right_cost[k] = 0;
      V3<R> amin(FMAX, FMAX, FMAX), amax(FMIN, FMIN, FMIN);
      uint32_t an = 0;
      for (int k = NBIN - 1; k >= 1; k--) {
        amin = amin.vmin(bnlo[k]);
        amax = amax.vmax(bnhi[k]);
        an += bnn[k];
        right_cost[k - 1] = an > 0 ? area(amin, amax) * R(an) : R(0);
      }
      int best_cut = -1;
      R best_cost = FMAX;
      amin = V3<R>(FMAX, FMAX, FMAX);
      amax = V3<R>(FMIN, FMIN, FMIN);
      an = 0;
      for (int k = 0; k < NBIN - 1; k++) {
        amin = amin.vmin(bnlo[k]);
        amax = amax.vmax(bnhi[k]);
        an += bnn[k];
        if (an == 0 || an == (uint32_t)count) continue;
        R cost = area(amin, amax) * R(an) + right_cost[k];
        if (cost < best_cost) { best_cost = cost; best_cut = k; }
      }
      if (best_cut < 0) {
        mid = start + count / 2;
      } else {
        size_t i = 0, j = count;
        while (i < j) {
          if (bin_of(prims[start + i]) <= best_cut) {
            i++;
          } else {
            j--;
            std::swap(prims[start + i], prims[start + j]);
          }
        }
        mid = start + i;
      }
    }
    mid = std::min(std::max(mid, start + 1), end - 1);
    uint32_t left = build_node(prims, start, mid);
    uint32_t right = build_node(prims, mid, end);
    nodes[idx].a = left;
    nodes[idx].b = right;
    return idx;
  }

  // mesh.rs:407-426 — slab test, entry distance (0 when inside).
  static bool ray_aabb(const V3<R>& bmin, const V3<R>& bmax, const V3<R>& o, const V3<R>& inv_d, R tmax, R* out) {
    R t0 = 0, t1 = tmax;
    for (int axis = 0; axis < 3; axis++) {
      R inv = inv_d.get(axis);
      R ta = (bmin.get(axis) - o.get(axis)) * inv;
      R tb = (bmax.get(axis) - o.get(axis)) * inv;
      if (ta > tb) std::swap(ta, tb);
      t0 = std::fmax(t0, ta);
      t1 = std::fmin(t1, tb);
      if (t0 > t1) return false;
    }
    *out = t0;
    return true;
  }

  // mesh.rs:436-456 — Möller–Trumbore, both faces, the reference epsilons.
  static bool ray_tri_packed(const V3<R>& a, const V3<R>& e1, const V3<R>& e2, const V3<R>& o, const V3<R>& d, R* tout) {
    V3<R> p = d.cross(e2);
    R det = e1.dot(p);
    if (std::fabs(det) < R(1e-9)) return false;
    R inv = R(1) / det;
    V3<R> s = o - a;
    R u = s.dot(p) * inv;
    if (!(u >= R(-1e-6) && u <= R(1) + R(1e-6))) return false;
    V3<R> q = s.cross(e1);
    R v = d.dot(q) * inv;
    if (v < R(-1e-6) || u + v > R(1) + R(1e-6)) return false;
    R t = e2.dot(q) * inv;
    if (t > R(1e-5)) { *tout = t; return true; }
    return false;
  }

  // mesh.rs:484-541 — ORDERED closest-hit traversal, 64-entry stack of
  // (node, t_enter), near child on top, strict `<` (first found wins ties).
  // Returns the ORIGINAL triangle id.
  //
  // tie = true: the precision-independent near-tie rule. Among all hits, let
  // t_min be the nearest; the hits within t_min * (1 + 1e-6) are near-ties of
  // it, and the winner is the lowest (authored surface id, original triangle
  // id, t) among them — the rule segment_hits applies to crossings
  // (mesh.rs:583-602), made a function of the set of hits alone. The walk
  // keeps the exact t_min and the winner so far and culls beyond
  // t_min * (1 + 1e-6); when a nearer hit shrinks the window past the winner
  // while an earlier hit may still be inside, it walks once more with the
  // final window (`fixed`) and takes the lowest key in it. The CUDA walks do
  // the same, so both find the same hit whatever their trees and orders.
  bool raycast(const V3<R>& o, const V3<R>& d, R* tout, uint32_t* triout, TraversalStats* st = nullptr,
               bool tie = false) const {
    if (nodes.empty()) return false;
    V3<R> inv_d(R(1) / d.x, R(1) / d.y, R(1) / d.z);
    const R rel = R(1e-6f);
    const R RMAX = R(std::numeric_limits<float>::max());
    bool have = false, fixed = false, amb = false;
    R bt = 0, bcull = RMAX, tmin = RMAX;
    uint32_t btri = 0, bsurf = 0;
    auto key_less = [](uint32_t as, uint32_t atr, R at, uint32_t bs, uint32_t btr, R btt) {
      return as < bs || (as == bs && (atr < btr || (atr == btr && at < btt)));
    };
    if (st) { st->queries++; st->unique_nodes++; }
    for (int pass = 0; pass < 2; pass++) {
      uint32_t sn[64];
      R stt[64];
      size_t sp = 1;
      sn[0] = 0; stt[0] = 0;
      while (sp > 0) {
        sp--;
        uint32_t ni = sn[sp];
        R t_enter = stt[sp];
        if (tie ? t_enter > bcull : (have && t_enter >= bt)) continue;
        const BvhNode<R>& node = nodes[ni];
        if (st) st->node_reads++;
        if (node.a & LEAF_BIT) {
          if (st) st->leaf_visits++;
          uint32_t start = node.a & ~LEAF_BIT;
          for (uint32_t i = start; i < start + node.b; i++) {
            const PackedTri<R>& pt = packed[i];
            if (st) st->prim_tests++;
            R t;
            if (ray_tri_packed(pt.a, pt.e1, pt.e2, o, d, &t)) {
              bool take;
              const uint32_t s = tri_surface[pt.tri];
              if (!tie) {
                take = !have || t < bt;
              } else if (fixed) {
                take = t <= bcull && (!have || key_less(s, pt.tri, t, bsurf, btri, bt));
              } else if (!have) {
                take = true;
                tmin = t;
              } else if (t < tmin) {
                const R win = t * (R(1) + rel);
                if (bt <= win) {
                  take = key_less(s, pt.tri, t, bsurf, btri, bt);
                } else {
                  if (tmin <= win) amb = true;
                  take = true;
                }
                tmin = t;
              } else {
                take = t <= bcull && key_less(s, pt.tri, t, bsurf, btri, bt);
              }
              if (tie && !fixed) bcull = tmin * (R(1) + rel);
              if (take) {
                have = true;
                bt = t;
                btri = pt.tri;
                bsurf = s;
                if (!tie) bcull = t;
              }
            }
          }
        } else {
          R tmax = (tie || have) ? bcull : RMAX;
          const BvhNode<R>& l = nodes[node.a];
          const BvhNode<R>& r = nodes[node.b];
          if (st) {
            st->node_reads += 2;
            st->internal_visits++;
            st->child_boxes += 2;
            // counted on the first pass only: exact for the reference's
            // one-pass walk; a near-tie walk's fixed-window second pass
            // re-reads (mostly) records the first pass touched
            if (pass == 0) st->unique_nodes += 2;
          }
          R ta, tb;
          bool hl, hr;
          if (tie) {
            const V3<R> g(tie_grow[0], tie_grow[1], tie_grow[2]);
            hl = ray_aabb(l.bmin - g, l.bmax + g, o, inv_d, tmax, &ta);
            hr = ray_aabb(r.bmin - g, r.bmax + g, o, inv_d, tmax, &tb);
          } else {
            hl = ray_aabb(l.bmin, l.bmax, o, inv_d, tmax, &ta);
            hr = ray_aabb(r.bmin, r.bmax, o, inv_d, tmax, &tb);
          }
          if (hl && hr) {
            uint32_t nearn, farn; R nt, ft;
            if (ta <= tb) { nearn = node.a; nt = ta; farn = node.b; ft = tb; }
            else { nearn = node.b; nt = tb; farn = node.a; ft = ta; }
            sn[sp] = farn; stt[sp] = ft;
            sn[sp + 1] = nearn; stt[sp + 1] = nt;
            sp += 2;
          } else if (hl) {
            sn[sp] = node.a; stt[sp] = ta; sp++;
          } else if (hr) {
            sn[sp] = node.b; stt[sp] = tb; sp++;
          }
        }
      }
      if (!tie || !amb || fixed) break;
      fixed = true;
      bcull = tmin * (R(1) + rel);
      have = false;
    }
    if (have) { *tout = bt; *triout = btri; }
    return have;
  }

  // Brute force over the packed primitives, for the BVH test (mesh.rs:697-736).
  bool raycast_brute(const V3<R>& o, const V3<R>& d, R* tout, uint32_t* triout) const {
    bool have = false;
    R bt = 0; uint32_t btri = 0;
    for (uint32_t t = 0; t < (uint32_t)tri_count(); t++) {
      V3<R> a, b, c;
      tri_verts(t, &a, &b, &c);
      R tt;
      if (ray_tri_packed(a, b - a, c - a, o, d, &tt)) {
        if (!have || tt < bt) { have = true; bt = tt; btri = t; }
      }
    }
    if (have) { *tout = bt; *triout = btri; }
    return have;
  }

  // mesh.rs:546-604 — every crossing strictly inside a->b, sorted, with the
  // same-t cluster merge that keeps the lowest surface id.
  void segment_hits(const V3<R>& a, const V3<R>& b, std::vector<SegHit>& out, TraversalStats* st = nullptr) const {
    out.clear();
    if (nodes.empty()) return;
    V3<R> d = b - a;
    R len = d.length();
    if (len < R(1e-6)) return;
    V3<R> dn = d * (R(1) / len);
    V3<R> inv_d(R(1) / dn.x, R(1) / dn.y, R(1) / dn.z);
    uint32_t stack[64];
    size_t sp = 1;
    stack[0] = 0;
    struct H { R t; uint32_t tri; uint16_t mat; };
    std::vector<H> hs;
    if (st) st->queries++;
    while (sp > 0) {
      sp--;
      const BvhNode<R>& node = nodes[stack[sp]];
      // this walk tests each node's own box when it pops it: every record once
      if (st) { st->node_reads++; st->unique_nodes++; }
      R tdummy;
      if (!ray_aabb(node.bmin, node.bmax, a, inv_d, len, &tdummy)) continue;
      if (st) (node.a & LEAF_BIT) ? st->leaf_visits++ : st->internal_visits++;
      if (node.a & LEAF_BIT) {
        uint32_t start = node.a & ~LEAF_BIT;
        for (uint32_t i = start; i < start + node.b; i++) {
          const PackedTri<R>& pt = packed[i];
          if (st) st->prim_tests++;
          R t;
          if (ray_tri_packed(pt.a, pt.e1, pt.e2, a, dn, &t)) {
            R tt = t / len;
            if (tt > R(1e-4) && tt < R(1) - R(1e-4)) hs.push_back({tt, pt.tri, pt.material});
          }
        }
      } else {
        stack[sp] = node.a;
        stack[sp + 1] = node.b;
        sp += 2;
      }
    }
    // Rust's sort_by is stable; total_cmp orders like < for these finite values
    std::stable_sort(hs.begin(), hs.end(), [](const H& x, const H& y) { return x.t < y.t; });
    R tol = R(1e-4) / std::fmax(len, R(1));
    size_t w = 0;
    for (size_t i = 0; i < hs.size(); i++) {
      if (w > 0 && std::fabs(hs[i].t - hs[w - 1].t) < tol) {
        if (tri_surface[hs[i].tri] < tri_surface[hs[w - 1].tri]) {
          hs[w - 1].tri = hs[i].tri;
          hs[w - 1].mat = hs[i].mat;
        }
      } else {
        hs[w] = hs[i];
        w++;
      }
    }
    hs.resize(w);
    for (auto& h : hs) out.push_back({(double)h.t, h.tri, h.mat});
  }

  // mesh.rs:607-620 — normal of the ORIGINAL triangle, flipped against d.
  bool raycast_hit(const V3<R>& p, const V3<R>& d, GeomHit<R>* h, TraversalStats* st = nullptr, uint32_t* tri_out = nullptr,
                   bool tie = false) const {
    R t; uint32_t tri;
    if (!raycast(p, d, &t, &tri, st, tie)) return false;
    V3<R> n = tri_normal(tri);
    if (n.dot(d) > R(0)) n = n * R(-1);
    h->t = t;
    h->normal = n;
    h->material = &materials[tri_material[tri]];
    if (tri_out) *tri_out = tri;
    return true;
  }
};

template <class R>
Mesh<R> mesh_from_builder(const MeshBuilder& mb) {   // mesh.rs:155-221
  Mesh<R> m;
  size_t nv = mb.positions.size() / 3;
  m.positions.resize(nv);
  for (size_t i = 0; i < nv; i++) m.positions[i] = from_f<R>(&mb.positions[3 * i]);
  m.indices = mb.indices;
  m.tri_material = mb.tri_material;
  m.materials = mb.materials;
  m.tri_surface = mb.tri_surface;
  m.tri_max_edge = mb.tri_max_edge;
  m.build_bvh();
  return m;
}

// scene.rs:94-137 — nearest of the base hit and each panel's slab entry.
template <class R, class G>
bool with_panels_hit(const G& base, const std::vector<BoxPanel<R>>& panels, const V3<R>& p, const V3<R>& d,
                     GeomHit<R>* best, TraversalStats* st = nullptr) {
  bool have = base.raycast_hit(p, d, best, st);
  const R FMAX = R(std::numeric_limits<float>::max());
  for (const BoxPanel<R>& pn : panels) {
    R t0 = 0, t1 = FMAX;
    int axis = 3;
    for (int a = 0; a < 3; a++) {
      R da = d.get(a), pa = p.get(a), lo = pn.mn.get(a), hi = pn.mx.get(a);
      if (std::fabs(da) < R(1e-9)) {
        if (pa < lo || pa > hi) { t0 = FMAX; break; }
      } else {
        R ta = (lo - pa) / da, tb = (hi - pa) / da;
        if (ta > tb) std::swap(ta, tb);
        if (ta > t0) { t0 = ta; axis = a; }
        t1 = std::fmin(t1, tb);
        if (t0 > t1) { t0 = FMAX; break; }
      }
    }
    if (t0 > R(1e-4) && t0 < FMAX && axis < 3 && (!have || t0 < best->t)) {
      V3<R> n(0, 0, 0);
      n.set(axis, d.get(axis) > R(0) ? R(-1) : R(1));
      best->t = t0;
      best->normal = n;
      best->material = &pn.m;
      have = true;
    }
  }
  return have;
}

// --------------------------------------------------------------- tracer
struct TraceParams {
  uint32_t n_bands = 3;         // lib.rs:22 NBANDS
  uint32_t n_bins = 300;        // tracer.rs:14
  float bin_dt = 0.010f;        // tracer.rs:12
  float max_time = 3.0f;        // tracer.rs:13
  uint32_t max_bounces = 64;    // tracer.rs:103
  float energy_floor = 1e-7f;   // tracer.rs:163,179 (relative to per-ray energy)
  float receiver_radius = 0.5f; // tracer.rs:15
  float wall_eps = 1e-3f;       // tracer.rs:16
  float speed_of_sound = 343.0f;// lib.rs:18
  uint32_t dir_band = 1;        // tracer.rs:123-125 (mid band)
  uint32_t tie_mode = 0;        // 0: reference first-found; 1: lowest surface id among near-ties
};

struct TraceStats {
  uint64_t segments = 0;        // bounce-loop iterations (tracer.rs:103-200)
  uint64_t receiver_hits = 0;
  TraversalStats trav;
};

// tracer.rs:80-202, one ray. `Hit` is any callable (p, d, GeomHit*) -> bool.
// Accumulates into bins (n_bins x n_bands) and dirs (n_bins x 3) of type A.
template <class R, class A, class G, class HitFn>
void trace_ray(HitFn&& hitfn, const TraceParams& P, const V3<R>& source, const V3<R>& listener,
               R per_ray, const float* source_energy, G& rng, A* bins, A* dirs, TraceStats* st,
               std::vector<uint32_t>* log_tri = nullptr, std::vector<float>* log_seg = nullptr) {
  const int NB = (int)P.n_bands;
  const R C = R(P.speed_of_sound);
  const R BIN_DT = R(P.bin_dt);
  const R MAX_TIME = R(P.max_time);
  const R WALL_EPS = R(P.wall_eps);
  const R RR = R(P.receiver_radius);
  const R floor_e = R(P.energy_floor) * per_ray;
  V3<R> pos = source;
  V3<R> dir = unit_sphere<R>(rng);
  R energy[MAXB];
  for (int b = 0; b < NB; b++) energy[b] = per_ray * R(source_energy[b]);
  R dist_total = 0;
  for (uint32_t bounce = 0; bounce < P.max_bounces; bounce++) {
    GeomHit<R> hit;
    uint32_t tri = 0xFFFFFFFFu;
    bool have = hitfn(pos, dir, &hit, &tri, st ? &st->trav : nullptr);
    if (st) st->segments++;
    if (log_seg) {
      log_seg->push_back((float)pos.x); log_seg->push_back((float)pos.y); log_seg->push_back((float)pos.z);
      log_seg->push_back((float)dir.x); log_seg->push_back((float)dir.y); log_seg->push_back((float)dir.z);
    }
    if (log_tri) log_tri->push_back(have ? tri : 0xFFFFFFFFu);
    R t_hit = have ? hit.t : R(std::numeric_limits<float>::max());
    V3<R> to_l = listener - pos;
    R s = to_l.dot(dir);
    if (s > R(0) && s < t_hit) {
      V3<R> closest = pos + dir * s;
      if ((closest - listener).length() < RR) {
        R arrival = (dist_total + s) / C;
        uint64_t bin = sat_u64<R>(arrival / BIN_DT);
        if (bin < P.n_bins) {
          if (st) st->receiver_hits++;
          for (int b = 0; b < NB; b++) bins[bin * NB + b] += (A)energy[b];
          R em = energy[P.dir_band];
          dirs[bin * 3 + 0] -= (A)(dir.x * em);
          dirs[bin * 3 + 1] -= (A)(dir.y * em);
          dirs[bin * 3 + 2] -= (A)(dir.z * em);
        }
      }
    }
    if (!have) break;
    pos = pos + dir * t_hit;
    dist_total += t_hit;
    if (dist_total / C > MAX_TIME) break;
    const Material& mat = *hit.material;
    R p_t = 0;
    for (int b = 0; b < NB; b++) {
      R tb = R(mat.transmission[b]);
      p_t = std::fmax(p_t, tb * tb);
    }
    R p = p_t > R(1e-5) ? std::fmin(std::fmax(p_t, R(0.02)), R(0.5)) : R(0);
    bool transmitted = p > R(0) && R(rng.next_f32()) < p;
    bool alive = false;
    if (transmitted) {
      for (int b = 0; b < NB; b++) {
        R tb = R(mat.transmission[b]);
        energy[b] *= (tb * tb) / p;
        if (energy[b] > floor_e) alive = true;
      }
      if (!alive) break;
      pos = pos + dir * (R(2) * WALL_EPS);
      continue;
    }
    for (int b = 0; b < NB; b++) {
      R tb = R(mat.transmission[b]);
      R keep = std::fmax(R(1) - R(mat.absorption[b]) - tb * tb, R(0));
      energy[b] *= keep / (R(1) - p);
      if (energy[b] > floor_e) alive = true;
    }
    if (!alive) break;
    V3<R> normal = hit.normal;
    if (R(rng.next_f32()) < R(mat.scattering)) {
      dir = (normal + unit_sphere<R>(rng)).normalize();
      if (dir.dot(normal) < R(1e-3)) dir = normal;
    } else {
      dir = dir - normal * (R(2) * dir.dot(normal));
    }
    pos = pos + normal * WALL_EPS;
  }
}

// --------------------------------------------------------------- reverb
// tracer.rs:204-257 — FP64 Schroeder integral, first bins at <= -5 and
// <= -25 dB, rt60 = clamp(-60 dt / ddB, 0.1, 5); late level = sqrt of the
// energy after 80 ms, capped at 0.7. Also a least-squares T20 fit of the
// EDC between those two bins (an addition; the 2-point slope is the parity
// definition).
template <class BinT, class LevelSumT>
void estimate_reverb(const BinT* bins, uint32_t n_bins, uint32_t nb, float bin_dt, float* rt60, float* level,
                     double* rt60_fit) {
  std::vector<double> edc(n_bins);
  for (uint32_t b = 0; b < nb; b++) {
    rt60[b] = 0.5f;
    if (rt60_fit) rt60_fit[b] = 0.5;
    double total = 0.0;
    for (int64_t i = (int64_t)n_bins - 1; i >= 0; i--) {
      total += (double)bins[i * nb + b];
      edc[i] = total;
    }
    if (total <= 0.0) continue;
    auto db = [&](uint32_t i) { return 10.0 * std::log10(std::fmax(edc[i] / total, 1e-12)); };
    int64_t t5 = -1, t25 = -1;
    for (uint32_t i = 0; i < n_bins; i++) {
      double d = db(i);
      if (t5 < 0 && d <= -5.0) t5 = i;
      if (t25 < 0 && d <= -25.0) { t25 = i; break; }
    }
    if (t5 >= 0 && t25 >= 0 && t25 > t5) {
      float dt = (float)(t25 - t5) * bin_dt;
      float ddb = (float)(db((uint32_t)t25) - db((uint32_t)t5));
      float r = -60.0f * dt / ddb;
      rt60[b] = std::fmin(std::fmax(r, 0.1f), 5.0f);
      if (rt60_fit) {
        double sx = 0, sy = 0, sxx = 0, sxy = 0, n = 0;
        for (int64_t i = t5; i <= t25; i++) {
          double x = (double)i * (double)bin_dt, y = db((uint32_t)i);
          sx += x; sy += y; sxx += x * x; sxy += x * y; n += 1;
        }
        double den = n * sxx - sx * sx;
        if (den > 0) {
          double slope = (n * sxy - sx * sy) / den;
          if (slope < 0) rt60_fit[b] = std::fmin(std::fmax(-60.0 / slope, 0.1), 5.0);
        }
      }
    }
  }
  uint64_t late_start = sat_u64<float>(0.080f / bin_dt);
  for (uint32_t b = 0; b < nb; b++) {
    LevelSumT late_e = 0;
    for (uint64_t i = late_start; i < n_bins; i++) late_e += (LevelSumT)bins[i * nb + b];
    level[b] = (float)std::fmin((double)std::sqrt(late_e), 0.7);
  }
}

// tracer.rs:62-77 — aggregate late direction and anisotropy (mid band).
template <class A>
void late_direction(const A* bins, const A* dirs, uint32_t n_bins, uint32_t nb, uint32_t mid, float bin_dt,
                    float from_s, float out_dir[3], float* aniso) {
  uint64_t start = sat_u64<float>(from_s / bin_dt);
  A v[3] = {0, 0, 0};
  A e = 0;
  for (uint64_t i = std::min<uint64_t>(start, n_bins); i < n_bins; i++) {
    for (int k = 0; k < 3; k++) v[k] += dirs[i * 3 + k];
    e += bins[i * nb + mid];
  }
  A len = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (len < A(1e-12) || e < A(1e-12)) {
    out_dir[0] = 1; out_dir[1] = 0; out_dir[2] = 0; *aniso = 0;
    return;
  }
  out_dir[0] = (float)(v[0] / len); out_dir[1] = (float)(v[1] / len); out_dir[2] = (float)(v[2] / len);
  *aniso = (float)std::fmin(len / e, A(1));
}

// ----------------------------------------------------------------- dome
// crates/omg-scene/src/dome.rs. The dome panel carries its own per-band
// amplitude transmission (the reference reads glass_transmission(heavy) or
// the door/heavy leaf constants, walkthrough.rs:310-326; callers pass those).
struct DomePanel {
  int axis;            // 0: plane of constant x, 1: constant y
  float plane;
  float lat0, lat1, z0, z1;
  int glass;           // 1: pane (transmits), 0: door leaf (blocks)
  float trans[MAXB];   // amplitude transmission (pane, or leaf seep)
};

template <class R>
bool dome_panel_hit(const DomePanel& pn, const V3<R>& o, const V3<R>& d, R t_max, R* tout) {  // dome.rs:56-68
  R po = pn.axis == 0 ? o.x : o.y, pd = pn.axis == 0 ? d.x : d.y;
  if (std::fabs(pd) < R(1e-8)) return false;
  R t = (R(pn.plane) - po) / pd;
  if (t < R(1e-4) || t >= t_max) return false;
  R lat = pn.axis == 0 ? o.y + t * d.y : o.x + t * d.x;
  R z = o.z + t * d.z;
  if (lat > R(pn.lat0) && lat < R(pn.lat1) && z > R(pn.z0) && z < R(pn.z1)) { *tout = t; return true; }
  return false;
}

// dome.rs:304-310 — 8 azimuth sectors + zenith.
template <class R>
int dome_bin_of(const V3<R>& d) {
  const float PI = 3.14159265358979323846f;
  const float TAU = 6.28318530717958647692f;
  if (d.z > R(0.87)) return 8;
  R az = R((float)std::atan2((double)d.y, (double)d.x)) + R(PI);
  uint64_t k = sat_u64<R>(az / (R(TAU) / R(8)));
  return (int)std::min<uint64_t>(k, 7);
}

// dome.rs:313-324 — golden-spiral fan.
template <class R>
std::vector<V3<R>> dome_fan(uint32_t n) {
  const float PI = 3.14159265358979323846f;
  R ga = R(PI) * (R(3) - std::sqrt(R(5)));
  std::vector<V3<R>> dirs(n);
  for (uint32_t i = 0; i < n; i++) {
    R z = R(1) - R(2) * (R(i) + R(0.5)) / R(n);
    R r = std::sqrt(std::fmax(R(1) - z * z, R(0)));
    R phi = ga * R(i);
    R s, c;
    sincos_r<R>(phi, &s, &c);
    dirs[i] = V3<R>(r * c, r * s, z);
  }
  return dirs;
}

struct DomeStats {
  uint64_t escape_events = 0;   // trace_escape loop iterations
  uint64_t through_calls = 0;   // trace_through calls
  TraversalStats trav;
};

// dome.rs:328-382 — specular escape, <= max_events, horizon 80 m.
template <class R>
bool dome_trace_escape(const Mesh<R>& mesh, const std::vector<DomePanel>& glass, const std::vector<DomePanel>& leaves,
                       V3<R> pos, V3<R> dir, uint32_t max_events, uint32_t nb, R* tp, DomeStats* st,
                       bool tie = false) {
  const R HORIZON = R(80);
  for (uint32_t b = 0; b < nb; b++) tp[b] = R(1);
  for (uint32_t ev = 0; ev < max_events; ev++) {
    if (st) st->escape_events++;
    R tm; uint32_t tri;
    bool mh = mesh.raycast(pos, dir, &tm, &tri, st ? &st->trav : nullptr, tie);
    R t_mesh = mh ? tm : R(std::numeric_limits<float>::max());
    R t_pan = t_mesh;
    const DomePanel* pan = nullptr;
    for (size_t k = 0; k < glass.size() + leaves.size(); k++) {
      const DomePanel& p = k < glass.size() ? glass[k] : leaves[k - glass.size()];
      R t;
      if (dome_panel_hit<R>(p, pos, dir, t_pan, &t)) { t_pan = t; pan = &p; }
    }
    if (pan) {
      if (!pan->glass) return false;
      for (uint32_t b = 0; b < nb; b++) tp[b] *= R(pan->trans[b]) * R(pan->trans[b]);
      pos = pos + dir * (t_pan + R(1e-3));
      continue;
    }
    auto escaped = [](const V3<R>& p, const V3<R>& d) { return p.z > R(-0.05) || d.z > R(0.05); };
    if (!mh) return escaped(pos, dir);
    if (tm > HORIZON) return escaped(pos, dir);
    const Material& m = mesh.materials[mesh.tri_material[tri]];
    for (uint32_t b = 0; b < nb; b++) tp[b] *= R(1) - R(m.absorption[b]);
    if (tp[1] < R(2e-3)) return false;
    V3<R> n = mesh.tri_normal(tri);
    V3<R> n_o = dir.dot(n) > R(0) ? n * R(-1) : n;
    V3<R> hit = pos + dir * tm;
    dir = (dir - n * (R(2) * dir.dot(n))).normalize();
    pos = hit + n_o * R(1e-3);
  }
  return false;
}

// dome.rs:384-422 — straight-through mass-law seep over a 50 m segment.
template <class R>
void dome_trace_through(const Mesh<R>& mesh, const std::vector<DomePanel>& glass, const std::vector<DomePanel>& leaves,
                        const V3<R>& eye, const V3<R>& dir, uint32_t nb, R* tp, std::vector<SegHit>& buf, DomeStats* st) {
  if (st) st->through_calls++;
  V3<R> end = eye + dir * R(50);
  for (uint32_t b = 0; b < nb; b++) tp[b] = R(1);
  if (end.z < R(-0.05)) { for (uint32_t b = 0; b < nb; b++) tp[b] = 0; return; }
  mesh.segment_hits(eye, end, buf, st ? &st->trav : nullptr);
  for (const SegHit& h : buf) {
    const Material& m = mesh.materials[h.material];
    for (uint32_t b = 0; b < nb; b++) tp[b] *= R(m.transmission[b]) * R(m.transmission[b]);
    if (tp[0] < R(1e-7)) { for (uint32_t b = 0; b < nb; b++) tp[b] = 0; return; }
  }
  for (size_t k = 0; k < glass.size() + leaves.size(); k++) {
    const DomePanel& p = k < glass.size() ? glass[k] : leaves[k - glass.size()];
    R t;
    if (dome_panel_hit<R>(p, eye, dir, R(80), &t)) {
      for (uint32_t b = 0; b < nb; b++) tp[b] *= R(p.trans[b]) * R(p.trans[b]);
    }
  }
}

// dome.rs:424-478 — one estimate: escape first, through when the escape is
// not near-full, per-band max, bin, EMA (1.0 on the first call).
template <class R>
void dome_sample(const Mesh<R>& mesh, const std::vector<DomePanel>& glass, const std::vector<DomePanel>& leaves,
                 const std::vector<V3<R>>& fan, const V3<R>& eye, uint32_t n_rays, uint32_t max_events, uint32_t nb,
                 float ema_alpha, float* ema_state /*9*nb*/, int* primed, float* out_dir /*9*3*/,
                 float* out_energy /*9*nb*/, double* raw_energy /*9*nb, before the EMA*/, uint8_t* escape_flags,
                 float* ray_tp /*n_rays*nb*/, DomeStats* st, bool tie = false) {
  const float PI = 3.14159265358979323846f;
  const float TAU = 6.28318530717958647692f;
  uint32_t N = (uint32_t)fan.size();
  R e[9][MAXB];
  V3<R> dsum[9];
  for (int k = 0; k < 9; k++) for (int b = 0; b < MAXB; b++) e[k][b] = 0;
  std::vector<SegHit> buf;
  for (uint32_t j = 0; j < n_rays; j++) {
    uint32_t i = (uint32_t)((uint64_t)j * N / n_rays);
    V3<R> d0 = fan[i];
    R bp[MAXB], tp[MAXB];
    bool esc = dome_trace_escape<R>(mesh, glass, leaves, eye, d0, max_events, nb, bp, st, tie);
    if (escape_flags) escape_flags[j] = esc ? 1 : 0;
    if (esc && bp[0] > R(0.5)) {
      for (uint32_t b = 0; b < nb; b++) tp[b] = bp[b];
    } else {
      dome_trace_through<R>(mesh, glass, leaves, eye, d0, nb, tp, buf, st);
      if (esc) for (uint32_t b = 0; b < nb; b++) tp[b] = std::fmax(tp[b], bp[b]);
    }
    if (ray_tp) for (uint32_t b = 0; b < nb; b++) ray_tp[j * nb + b] = (float)tp[b];
    if (tp[0] > R(1e-9)) {
      int bi = dome_bin_of<R>(d0);
      for (uint32_t b = 0; b < nb; b++) e[bi][b] += tp[b] / R(n_rays);
      dsum[bi] = dsum[bi] + d0 * std::fmax(tp[1], tp[0] * R(0.2));
    }
  }
  float alpha = *primed ? ema_alpha : 1.0f;
  *primed = 1;
  for (int k = 0; k < 9; k++) {
    for (uint32_t b = 0; b < nb; b++) {
      if (raw_energy) raw_energy[k * nb + b] = (double)e[k][b];
      ema_state[k * nb + b] += alpha * ((float)e[k][b] - ema_state[k * nb + b]);
      out_energy[k * nb + b] = ema_state[k * nb + b];
    }
    V3<R> d;
    if (dsum[k].length() > R(1e-6)) {
      d = dsum[k].normalize();
    } else {
      R az = (R(k) + R(0.5)) * R(TAU) / R(8) - R(PI);
      R s, c;
      sincos_r<R>(az, &s, &c);
      d = k == 8 ? V3<R>(0, 0, 1) : V3<R>(c, s, 0);
    }
    out_dir[k * 3 + 0] = (float)d.x;
    out_dir[k * 3 + 1] = (float)d.y;
    out_dir[k * 3 + 2] = (float)d.z;
  }
}

}  // namespace orc

namespace orc {

// ----------------------------------------------------------- world build
// crates/omg-scene/src/dome.rs:79-119 — rectangle minus holes as sub-rectangles.
struct Rect { float u0, u1, v0, v1; };

inline std::vector<Rect> subrects(Rect r, const std::vector<Rect>& holes) {
  std::vector<float> cuts{r.u0, r.u1};
  for (const Rect& h : holes) {
    cuts.push_back(std::fmin(std::fmax(h.u0, r.u0), r.u1));
    cuts.push_back(std::fmin(std::fmax(h.u1, r.u0), r.u1));
  }
  std::stable_sort(cuts.begin(), cuts.end());
  std::vector<float> ded;
  for (float c : cuts) {
    if (!ded.empty() && std::fabs(c - ded.back()) < 1e-4f) continue;  // Vec::dedup_by keeps the first
    ded.push_back(c);
  }
  std::vector<Rect> out;
  for (size_t k = 0; k + 1 < ded.size(); k++) {
    float u0 = ded[k], u1 = ded[k + 1];
    if (u1 - u0 < 1e-3f) continue;
    float um = 0.5f * (u0 + u1);
    std::vector<std::pair<float, float>> vh;
    for (const Rect& h : holes) {
      if (h.u0 <= um && um <= h.u1) {
        float a = std::fmax(h.v0, r.v0), b = std::fmin(h.v1, r.v1);
        if (b > a) vh.push_back({a, b});
      }
    }
    std::stable_sort(vh.begin(), vh.end(), [](const std::pair<float, float>& x, const std::pair<float, float>& y) {
      return x.first < y.first;
    });
    float v = r.v0;
    for (auto& h : vh) {
      if (h.first - v > 1e-3f) out.push_back({u0, u1, v, h.first});
      v = std::fmax(v, h.second);
    }
    if (r.v1 - v > 1e-3f) out.push_back({u0, u1, v, r.v1});
  }
  return out;
}

struct RoomC {       // walkthrough.rs:29-42
  float min[2], max[2];
  float height, barrier_height, floor_z, wall_thickness;
  int outdoor;
  Material walls[6];
};

struct DoorC {       // walkthrough.rs:228-249 (+ pane transmission)
  int rooms[2];
  float pos[2];
  int axis;
  float half, height, zc;
  int glass;
  float openness;
  int heavy;
  float pane_trans[MAXB];
};

// material.rs:59-62 in f32
inline Material with_thickness(const Material& m, float thickness, int nb) {
  Material o = m;
  float k = std::fmin(0.15f / std::fmax(thickness, 0.02f), 2.0f);
  for (int b = 0; b < nb; b++) o.transmission[b] = std::fmin(m.transmission[b] * k, 0.9f);
  return o;
}

// dome.rs:121-258 — the world mesh: ground (coarse outside the town band),
// every room's walls with true holes, ceiling slabs with stairwell holes.
// Returns the glass panes as dome panels.
inline std::vector<DomePanel> build_world_mesh(MeshBuilder& b, const std::vector<RoomC>& rooms,
                                               const std::vector<DoorC>& doors, float town0, float town1,
                                               float wall_max_edge, int nb) {
  std::vector<DomePanel> glass;
  const RoomC* outdoor = nullptr;
  for (const RoomC& r : rooms) if (r.outdoor) { outdoor = &r; break; }
  if (!outdoor) return glass;
  uint16_t ground = b.material(outdoor->walls[4]);
  b.begin_surface();
  std::vector<Rect> shafts;
  for (const DoorC& d : doors)
    if (d.zc < 0.0f) shafts.push_back({d.pos[0] - 1.5f, d.pos[0] + 0.8f, d.pos[1] - d.half, d.pos[1] + d.half});
  for (const Rect& s : subrects({outdoor->min[0], outdoor->max[0], outdoor->min[1], outdoor->max[1]}, shafts)) {
    struct Band { float y0, y1, coarse; };
    std::vector<Band> bands;
    float n0 = std::fmax(s.v0, town0), n1 = std::fmin(s.v1, town1);
    if (s.v0 < town0) bands.push_back({s.v0, std::fmin(s.v1, town0), 64.0f});
    if (n1 > n0) bands.push_back({n0, n1, 0.0f});
    if (s.v1 > town1) bands.push_back({std::fmax(s.v0, town1), s.v1, 64.0f});
    for (const Band& bd : bands) {
      b.coarse(bd.coarse == 0.0f ? wall_max_edge : bd.coarse);
      float A[3] = {s.u0, bd.y0, 0.0f}, B[3] = {s.u1, bd.y0, 0.0f}, Cc[3] = {s.u1, bd.y1, 0.0f},
            D[3] = {s.u0, bd.y1, 0.0f};
      b.quad(A, B, Cc, D, ground);
    }
    b.coarse(wall_max_edge);
  }
  for (size_t ri = 0; ri < rooms.size(); ri++) {
    const RoomC& r = rooms[ri];
    if (r.outdoor) continue;
    float z0 = r.floor_z, z1 = r.floor_z + r.height;
    const RoomC* above = nullptr;
    for (const RoomC& n : rooms) {
      if (!n.outdoor && n.floor_z >= z1 - 0.05f && n.floor_z <= z1 + 0.8f && std::fabs(n.min[0] - r.min[0]) < 2.0f &&
          std::fabs(n.min[1] - r.min[1]) < 2.0f) {
        above = &n;
        break;
      }
    }
    float wall_top = above ? above->floor_z : std::fmax(r.barrier_height, z1);
    struct Side { int wi; float plane, lo, hi; int axis; };
    const Side sides[4] = {{0, r.min[0], r.min[1], r.max[1], 0}, {1, r.max[0], r.min[1], r.max[1], 0},
                           {2, r.min[1], r.min[0], r.max[0], 1}, {3, r.max[1], r.min[0], r.max[0], 1}};
    for (const Side& sd : sides) {
      uint16_t mat = b.material(with_thickness(r.walls[sd.wi], r.wall_thickness, nb));
      b.begin_surface();
      std::vector<Rect> holes;
      for (const DoorC& d : doors) {
        if (d.axis != sd.axis || (d.rooms[0] != (int)ri && d.rooms[1] != (int)ri)) continue;
        float dp = sd.axis == 0 ? d.pos[0] : d.pos[1];
        float dl = sd.axis == 0 ? d.pos[1] : d.pos[0];
        if (std::fabs(dp - sd.plane) > 0.1f) continue;
        holes.push_back({dl - d.half, dl + d.half, d.zc - 0.5f * d.height, d.zc + 0.5f * d.height});
        if (d.glass) {
          DomePanel p;
          std::memset(&p, 0, sizeof(p));
          p.axis = sd.axis;
          p.plane = sd.plane;
          p.lat0 = dl - d.half;
          p.lat1 = dl + d.half;
          p.z0 = d.zc - 0.5f * d.height;
          p.z1 = d.zc + 0.5f * d.height;
          p.glass = 1;
          for (int k = 0; k < nb; k++) p.trans[k] = d.pane_trans[k];
          glass.push_back(p);
        }
      }
      for (const Rect& s : subrects({sd.lo, sd.hi, z0, wall_top}, holes)) {
        auto P = [&](float u, float v, float* o) {
          if (sd.axis == 0) { o[0] = sd.plane; o[1] = u; o[2] = v; }
          else { o[0] = u; o[1] = sd.plane; o[2] = v; }
        };
        float A[3], B[3], Cc[3], D[3];
        P(s.u0, s.v0, A); P(s.u1, s.v0, B); P(s.u1, s.v1, Cc); P(s.u0, s.v1, D);
        b.quad(A, B, Cc, D, mat);
      }
    }
    uint16_t mat = b.material(with_thickness(r.walls[5], r.wall_thickness, nb));
    b.begin_surface();
    std::vector<Rect> holes;
    for (const DoorC& d : doors) {
      bool vertical = std::fabs(d.zc - z1) < 0.6f;
      if (vertical && (d.rooms[0] == (int)ri || d.rooms[1] == (int)ri) && !d.glass)
        holes.push_back({d.pos[0] - d.half, d.pos[0] + d.half, d.pos[1] - d.half, d.pos[1] + d.half});
    }
    for (const Rect& s : subrects({r.min[0], r.max[0], r.min[1], r.max[1]}, holes)) {
      float A[3] = {s.u0, s.v0, z1}, B[3] = {s.u1, s.v0, z1}, Cc[3] = {s.u1, s.v1, z1}, D[3] = {s.u0, s.v1, z1};
      b.quad(A, B, Cc, D, mat);
    }
  }
  return glass;
}

}  // namespace orc
