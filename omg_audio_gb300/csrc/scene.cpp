// Host-side scene preparation: mesh builder with vertex dedup, tessellation of
// oversized triangles, the reference's binned-SAH BVH (and a three-axis binned
// SAH tree for near-tie walks), and flattening into the
// device layout (child-box BVH2, 48-byte primitives, per-triangle normals).
//
// Compiled with -ffp-contract=off: every f32 result here (midpoints, edges,
// boxes, normals) rounds exactly as the reference's Rust code does, so the
// SAH tree and the primitive list are bit-identical to mesh.rs's.
#include "scene.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>

namespace omg {

// ------------------------------------------------------------ mesh builder
// mesh.rs:70-165
uint32_t MeshBuilder::material(const omg_material& m) {
  materials.push_back(m);
  return (uint32_t)(materials.size() - 1);
}

uint32_t MeshBuilder::begin_surface() {
  next_surface++;
  return (uint32_t)(uint16_t)(next_surface - 1);
}

uint32_t MeshBuilder::vertex(const float p[3]) {
  // mesh.rs:108-114: quantise to 0.1 mm, f32 product, round half away from zero
  auto q = [](float v) { return (int64_t)std::round(v * 1e4f); };
  Key k{q(p[0]), q(p[1]), q(p[2])};
  auto it = lookup.find(k);
  if (it != lookup.end()) return it->second;
  uint32_t id = (uint32_t)(positions.size() / 3);
  positions.push_back(p[0]);
  positions.push_back(p[1]);
  positions.push_back(p[2]);
  lookup.emplace(k, id);
  return id;
}

void MeshBuilder::tri(const float a[3], const float b[3], const float c[3], uint32_t m) {
  uint32_t ia = vertex(a), ib = vertex(b), ic = vertex(c);
  indices.push_back(ia);
  indices.push_back(ib);
  indices.push_back(ic);
  tri_material.push_back((uint16_t)m);
  tri_surface.push_back(next_surface > 0 ? (uint16_t)(next_surface - 1) : (uint16_t)0);
  tri_max_edge.push_back(cur_max_edge > 0.0f ? cur_max_edge : kMaxPrimEdge);
}

void MeshBuilder::quad(const float a[3], const float b[3], const float c[3], const float d[3], uint32_t m) {
  tri(a, b, c, m);
  tri(a, c, d, m);
}

void MeshBuilder::abox(const float mn[3], const float mx[3], uint32_t m) {
  const float ax = mn[0], ay = mn[1], az = mn[2], bx = mx[0], by = mx[1], bz = mx[2];
  auto Q = [&](float p0, float p1, float p2, float q0, float q1, float q2, float r0, float r1, float r2, float s0,
               float s1, float s2) {
    const float A[3] = {p0, p1, p2}, B[3] = {q0, q1, q2}, Cc[3] = {r0, r1, r2}, D[3] = {s0, s1, s2};
    quad(A, B, Cc, D, m);
  };
  Q(ax, ay, az, ax, by, az, ax, by, bz, ax, ay, bz);
  Q(bx, ay, az, bx, ay, bz, bx, by, bz, bx, by, az);
  Q(ax, ay, az, ax, ay, bz, bx, ay, bz, bx, ay, az);
  Q(ax, by, az, bx, by, az, bx, by, bz, ax, by, bz);
  Q(ax, ay, az, bx, ay, az, bx, by, az, ax, by, az);
  Q(ax, ay, bz, ax, by, bz, bx, by, bz, bx, ay, bz);
}

// --------------------------------------------------------------- vec math
namespace {
struct F3 {
  float x, y, z;
};
inline F3 add(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline F3 sub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline F3 mul(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float len(F3 a) { return std::sqrt(dot(a, a)); }
inline F3 cross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline F3 vmin(F3 a, F3 b) { return {std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)}; }
inline F3 vmax(F3 a, F3 b) { return {std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)}; }
inline float get(F3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
inline F3 normalize(F3 a) {  // vec3.rs:19-26
  float l = len(a);
  if (l > 1e-12f) return mul(a, 1.0f / l);
  return {1.0f, 0.0f, 0.0f};
}

struct Prim {
  F3 a, e1, e2;
  uint32_t tri;
  uint16_t material;
  uint32_t id;    // tessellation index (carried, never compared)
};

struct RefNode {  // mesh.rs:52-58
  F3 bmin, bmax;
  uint32_t a, b;
};

constexpr uint32_t kLeafBit = 1u << 31;  // mesh.rs:17
constexpr size_t kLeafSize = 4;          // mesh.rs:16

inline void pbounds(const Prim& p, F3* lo, F3* hi) {
  F3 a = p.a, b = add(p.a, p.e1), c = add(p.a, p.e2);
  *lo = vmin(vmin(a, b), c);
  *hi = vmax(vmax(a, b), c);
}
inline F3 pcentroid(const Prim& p) { return add(p.a, mul(add(p.e1, p.e2), 1.0f / 3.0f)); }
inline float area(F3 lo, F3 hi) {
  F3 e = vmax(sub(hi, lo), F3{0, 0, 0});
  return 2.0f * (e.x * e.y + e.y * e.z + e.z * e.x);
}
inline uint64_t sat_u64(float v) {
  if (!(v >= 0.0f)) return 0;
  if (v >= 1.8446744073709552e19f) return UINT64_MAX;
  return (uint64_t)v;
}

// mesh.rs:292-405
uint32_t build_node(std::vector<RefNode>& nodes, std::vector<Prim>& prims, size_t start, size_t end) {
  const int NBIN = 16;
  const float FMAX = std::numeric_limits<float>::max();
  F3 bmin{FMAX, FMAX, FMAX}, bmax{-FMAX, -FMAX, -FMAX}, cmin = bmin, cmax = bmax;
  for (size_t i = start; i < end; i++) {
    F3 lo, hi;
    pbounds(prims[i], &lo, &hi);
    bmin = vmin(bmin, lo);
    bmax = vmax(bmax, hi);
    F3 c = pcentroid(prims[i]);
    cmin = vmin(cmin, c);
    cmax = vmax(cmax, c);
  }
  uint32_t idx = (uint32_t)nodes.size();
  nodes.push_back({bmin, bmax, 0, 0});
  size_t count = end - start;
  if (count <= kLeafSize) {
    nodes[idx].a = kLeafBit | (uint32_t)start;
    nodes[idx].b = (uint32_t)count;
    return idx;
  }
  F3 cext = sub(cmax, cmin);
  int axis = (cext.x >= cext.y && cext.x >= cext.z) ? 0 : (cext.y >= cext.z ? 1 : 2);
  float cwidth = get(cext, axis);
  size_t mid;
  if (cwidth < 1e-6f) {
    mid = start + count / 2;
  } else {
    const float cmin_a = get(cmin, axis);
    auto bin_of = [&](const Prim& p) -> int {
      float v = (get(pcentroid(p), axis) - cmin_a) / cwidth * (float)NBIN;
      v = std::fmin(v, (float)NBIN - 1.0f);
      return (int)sat_u64(v);
    };
    F3 blo[NBIN], bhi[NBIN];
    uint32_t bn[NBIN];
    for (int k = 0; k < NBIN; k++) {
      blo[k] = {FMAX, FMAX, FMAX};
      bhi[k] = {-FMAX, -FMAX, -FMAX};
      bn[k] = 0;
    }
    for (size_t i = start; i < end; i++) {
      int k = bin_of(prims[i]);
      F3 lo, hi;
      pbounds(prims[i], &lo, &hi);
      blo[k] = vmin(blo[k], lo);
      bhi[k] = vmax(bhi[k], hi);
      bn[k] += 1;
    }
    float right_cost[NBIN] = {0};
    F3 amin{FMAX, FMAX, FMAX}, amax{-FMAX, -FMAX, -FMAX};
    uint32_t an = 0;
    for (int k = NBIN - 1; k >= 1; k--) {
      amin = vmin(amin, blo[k]);
      amax = vmax(amax, bhi[k]);
      an += bn[k];
      right_cost[k - 1] = an > 0 ? area(amin, amax) * (float)an : 0.0f;
    }
    int best_cut = -1;
    float best_cost = FMAX;
    amin = {FMAX, FMAX, FMAX};
    amax = {-FMAX, -FMAX, -FMAX};
    an = 0;
    for (int k = 0; k < NBIN - 1; k++) {
      amin = vmin(amin, blo[k]);
      amax = vmax(amax, bhi[k]);
      an += bn[k];
      if (an == 0 || an == (uint32_t)count) continue;
      float cost = area(amin, amax) * (float)an + right_cost[k];
      if (cost < best_cost) {
        best_cost = cost;
        best_cut = k;
      }
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
  uint32_t left = build_node(nodes, prims, start, mid);
  uint32_t right = build_node(nodes, prims, mid, end);
  nodes[idx].a = left;
  nodes[idx].b = right;
  return idx;
}
}  // namespace

// mesh.rs:241-287 — tessellate (longest edge at its midpoint, LIFO work list).
void tessellate(const float* pos, const uint32_t* idx, uint32_t n_tris, const uint16_t* tri_mat,
                const float* tri_max_edge, std::vector<float>& prim_geo, std::vector<uint32_t>& prim_tri,
                std::vector<uint16_t>& prim_mat, std::vector<float>* prim_vtx) {
  struct W {
    F3 a, b, c;
    uint32_t t;
  };
  auto vtx = [&](uint32_t i) { return F3{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]}; };
  std::vector<W> work;
  work.reserve(n_tris);
  for (uint32_t t = 0; t < n_tris; t++) work.push_back({vtx(idx[3 * t]), vtx(idx[3 * t + 1]), vtx(idx[3 * t + 2]), t});
  prim_geo.clear();
  prim_tri.clear();
  prim_mat.clear();
  if (prim_vtx) prim_vtx->clear();
  while (!work.empty()) {
    W w = work.back();
    work.pop_back();
    F3 a = w.a, b = w.b, c = w.c;
    float lab = len(sub(b, a)), lbc = len(sub(c, b)), lca = len(sub(a, c));
    float longest = std::fmax(std::fmax(lab, lbc), lca);
    float lim = tri_max_edge ? tri_max_edge[w.t] : kMaxPrimEdge;
    if (longest > lim) {
      if (lab >= lbc && lab >= lca) {
        F3 m = mul(add(a, b), 0.5f);
        work.push_back({a, m, c, w.t});
        work.push_back({m, b, c, w.t});
      } else if (lbc >= lca) {
        F3 m = mul(add(b, c), 0.5f);
        work.push_back({a, b, m, w.t});
        work.push_back({a, m, c, w.t});
      } else {
        F3 m = mul(add(c, a), 0.5f);
        work.push_back({a, b, m, w.t});
        work.push_back({m, b, c, w.t});
      }
      continue;
    }
    F3 e1 = sub(b, a), e2 = sub(c, a);
    const float g[9] = {a.x, a.y, a.z, e1.x, e1.y, e1.z, e2.x, e2.y, e2.z};
    prim_geo.insert(prim_geo.end(), g, g + 9);
    if (prim_vtx) {
      const float v[9] = {a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z};
      prim_vtx->insert(prim_vtx->end(), v, v + 9);
    }
    prim_tri.push_back(w.t);
    prim_mat.push_back(tri_mat[w.t]);
  }
}

// Reference SAH tree over the tessellated prims (reorders them into leaf
// order). ref_boxes/ref_ab receive the reference's node array.
void build_sah(std::vector<float>& prim_geo, std::vector<uint32_t>& prim_tri, std::vector<uint16_t>& prim_mat,
               std::vector<float>& ref_boxes, std::vector<uint32_t>& ref_ab, std::vector<uint32_t>* perm) {
  size_t n = prim_tri.size();
  std::vector<Prim> prims(n);
  for (size_t i = 0; i < n; i++) {
    const float* g = &prim_geo[9 * i];
    prims[i] = {{g[0], g[1], g[2]}, {g[3], g[4], g[5]}, {g[6], g[7], g[8]}, prim_tri[i], prim_mat[i], (uint32_t)i};
  }
  std::vector<RefNode> nodes;
  ref_boxes.clear();
  ref_ab.clear();
  if (n == 0) return;
  nodes.reserve(2 * n / kLeafSize + 8);
  build_node(nodes, prims, 0, n);
  if (perm) perm->resize(n);
  for (size_t i = 0; i < n; i++) {
    const Prim& p = prims[i];
    if (perm) (*perm)[i] = p.id;
    const float g[9] = {p.a.x, p.a.y, p.a.z, p.e1.x, p.e1.y, p.e1.z, p.e2.x, p.e2.y, p.e2.z};
    std::memcpy(&prim_geo[9 * i], g, sizeof(g));
    prim_tri[i] = p.tri;
    prim_mat[i] = p.material;
  }
  ref_boxes.resize(nodes.size() * 6);
  ref_ab.resize(nodes.size() * 2);
  for (size_t i = 0; i < nodes.size(); i++) {
    const RefNode& r = nodes[i];
    float* o = &ref_boxes[6 * i];
    o[0] = r.bmin.x; o[1] = r.bmin.y; o[2] = r.bmin.z;
    o[3] = r.bmax.x; o[4] = r.bmax.y; o[5] = r.bmax.z;
    ref_ab[2 * i] = r.a;
    ref_ab[2 * i + 1] = r.b;
  }
}

// Binned SAH over all three axes (128 bins per axis, primitives binned by the
// centre of their box), leaves of at most 4 primitives. The reference bins
// only the widest centroid axis in 16 bins; on the 40-room scene this tree
// needs a third fewer node visits and a fifth fewer triangle tests per
// closest-hit query. The closest hit under the near-tie rule does not depend
// on the tree. Below depth 36 the split is the SAH one; deeper (degenerate
// inputs only) it is the object median of the widest axis, so a path never
// exceeds 36 + log2(n) < 64 nodes (the traversal stack depth).
namespace {
struct BinBox {
  float lo[3], hi[3];
  void clear() {
    for (int k = 0; k < 3; k++) {
      lo[k] = std::numeric_limits<float>::max();
      hi[k] = -std::numeric_limits<float>::max();
    }
  }
  void grow(const BinBox& o) {
    for (int k = 0; k < 3; k++) {
      lo[k] = std::fmin(lo[k], o.lo[k]);
      hi[k] = std::fmax(hi[k], o.hi[k]);
    }
  }
  float half_area() const {
    float e[3];
    for (int k = 0; k < 3; k++) e[k] = std::fmax(hi[k] - lo[k], 0.0f);
    return e[0] * e[1] + e[1] * e[2] + e[2] * e[0];
  }
};

struct SweepPrim {
  BinBox b;
  float c[3];
  uint32_t id;
};

struct Sah3Builder {
  static constexpr int kBins = 128;
  static constexpr int kMedianDepth = 36;
  std::vector<SweepPrim>& P;
  std::vector<BinBox> boxes;
  std::vector<uint32_t> ab;
  BinBox bins[3][kBins];
  uint32_t counts[3][kBins];
  float right_cost[kBins];

  explicit Sah3Builder(std::vector<SweepPrim>& p) : P(p) {}

  uint32_t node(size_t s, size_t e, int depth) {
    BinBox bb, cb;
    bb.clear();
    cb.clear();
    for (size_t i = s; i < e; i++) {
      bb.grow(P[i].b);
      for (int k = 0; k < 3; k++) {
        cb.lo[k] = std::fmin(cb.lo[k], P[i].c[k]);
        cb.hi[k] = std::fmax(cb.hi[k], P[i].c[k]);
      }
    }
    const uint32_t idx = (uint32_t)boxes.size();
    boxes.push_back(bb);
    ab.push_back(0);
    ab.push_back(0);
    const size_t n = e - s;
    if (n <= kLeafSize) {
      ab[2 * idx] = kLeafBit | (uint32_t)s;
      ab[2 * idx + 1] = (uint32_t)n;
      return idx;
    }
    int best_axis = -1, best_cut = -1;
    if (depth < kMedianDepth) {
      float best = std::numeric_limits<float>::max();
      for (int a = 0; a < 3; a++) {
        const float w = cb.hi[a] - cb.lo[a];
        if (!(w > 1e-6f)) continue;
        const float scale = (float)kBins / w;
        for (int k = 0; k < kBins; k++) {
          bins[a][k].clear();
          counts[a][k] = 0;
        }
        for (size_t i = s; i < e; i++) {
          const int k = std::min(kBins - 1, (int)((P[i].c[a] - cb.lo[a]) * scale));
          bins[a][k].grow(P[i].b);
          counts[a][k]++;
        }
        BinBox acc;
        acc.clear();
        uint32_t cnt = 0;
        for (int k = kBins - 1; k >= 1; k--) {
          acc.grow(bins[a][k]);
          cnt += counts[a][k];
          right_cost[k - 1] = cnt ? acc.half_area() * (float)cnt : 0.0f;
        }
        acc.clear();
        cnt = 0;
        for (int k = 0; k < kBins - 1; k++) {
          acc.grow(bins[a][k]);
          cnt += counts[a][k];
          if (cnt == 0 || cnt == n) continue;
          const float cost = acc.half_area() * (float)cnt + right_cost[k];
          if (cost < best) {
            best = cost;
            best_axis = a;
            best_cut = k;
          }
        }
      }
    }
    size_t mid;
    if (best_axis >= 0) {
      const int a = best_axis;
      const float scale = (float)kBins / (cb.hi[a] - cb.lo[a]), lo = cb.lo[a];
      auto it = std::partition(P.begin() + s, P.begin() + e, [&](const SweepPrim& p) {
        return std::min(kBins - 1, (int)((p.c[a] - lo) * scale)) <= best_cut;
      });
      mid = (size_t)(it - P.begin());
    } else {
      // object median of the widest centroid axis
      int a = 0;
      for (int k = 1; k < 3; k++)
        if (cb.hi[k] - cb.lo[k] > cb.hi[a] - cb.lo[a]) a = k;
      mid = s + n / 2;
      std::nth_element(P.begin() + s, P.begin() + mid, P.begin() + e,
                       [&](const SweepPrim& x, const SweepPrim& y) {
                         return x.c[a] < y.c[a] || (x.c[a] == y.c[a] && x.id < y.id);
                       });
    }
    if (mid <= s || mid >= e) mid = s + n / 2;
    const uint32_t l = node(s, mid, depth + 1);
    const uint32_t r = node(mid, e, depth + 1);
    ab[2 * idx] = l;
    ab[2 * idx + 1] = r;
    return idx;
  }
};
}  // namespace

void build_sah3(std::vector<float>& prim_geo, std::vector<uint32_t>& prim_tri, std::vector<uint16_t>& prim_mat,
                std::vector<float>& ref_boxes, std::vector<uint32_t>& ref_ab, std::vector<uint32_t>* perm) {
  const size_t n = prim_tri.size();
  ref_boxes.clear();
  ref_ab.clear();
  if (n == 0) return;
  std::vector<SweepPrim> P(n);
  for (size_t i = 0; i < n; i++) {
    const float* g = &prim_geo[9 * i];
    for (int k = 0; k < 3; k++) {
      const float x0 = g[k], x1 = g[k] + g[3 + k], x2 = g[k] + g[6 + k];
      P[i].b.lo[k] = std::fmin(std::fmin(x0, x1), x2);
      P[i].b.hi[k] = std::fmax(std::fmax(x0, x1), x2);
      P[i].c[k] = (P[i].b.lo[k] + P[i].b.hi[k]) * 0.5f;
    }
    P[i].id = (uint32_t)i;
  }
  std::unique_ptr<Sah3Builder> B(new Sah3Builder(P));
  B->boxes.reserve(2 * n / kLeafSize + 8);
  B->ab.reserve(4 * n / kLeafSize + 16);
  B->node(0, n, 0);
  std::vector<float> geo(prim_geo.size());
  std::vector<uint32_t> tri(n);
  std::vector<uint16_t> mat(n);
  if (perm) perm->resize(n);
  for (size_t i = 0; i < n; i++) {
    if (perm) (*perm)[i] = P[i].id;
    std::memcpy(&geo[9 * i], &prim_geo[9 * (size_t)P[i].id], 9 * sizeof(float));
    tri[i] = prim_tri[P[i].id];
    mat[i] = prim_mat[P[i].id];
  }
  prim_geo.swap(geo);
  prim_tri.swap(tri);
  prim_mat.swap(mat);
  ref_boxes.resize(B->boxes.size() * 6);
  for (size_t i = 0; i < B->boxes.size(); i++) {
    float* o = &ref_boxes[6 * i];
    const BinBox& b = B->boxes[i];
    o[0] = b.lo[0]; o[1] = b.lo[1]; o[2] = b.lo[2];
    o[3] = b.hi[0]; o[4] = b.hi[1]; o[5] = b.hi[2];
  }
  ref_ab.swap(B->ab);
}

// Flatten the reference node array into the device BVH2: one device node per
// internal reference node, holding both children's boxes; leaf children are
// encoded in the parent's child ref.
int32_t flatten_bvh2(const std::vector<float>& ref_boxes, const std::vector<uint32_t>& ref_ab,
                     std::vector<float>& dev_nodes) {
  size_t nref = ref_ab.size() / 2;
  dev_nodes.clear();
  if (nref == 0) return 0;
  auto leaf_code = [&](uint32_t i) -> int32_t {
    uint32_t start = ref_ab[2 * i] & ~kLeafBit, count = ref_ab[2 * i + 1];
    return (int32_t)~((start << 3) | (count - 1));
  };
  if (ref_ab[0] & kLeafBit) return leaf_code(0);
  std::vector<int32_t> dev_of(nref, -1);
  int32_t next = 0;
  // preorder numbering of internal nodes (root = 0)
  std::vector<uint32_t> st{0};
  std::vector<uint32_t> order;
  while (!st.empty()) {
    uint32_t i = st.back();
    st.pop_back();
    if (ref_ab[2 * i] & kLeafBit) continue;
    dev_of[i] = next++;
    order.push_back(i);
    st.push_back(ref_ab[2 * i + 1]);
    st.push_back(ref_ab[2 * i]);
  }
  dev_nodes.assign((size_t)next * 16, 0.0f);
  for (uint32_t i : order) {
    float* o = &dev_nodes[(size_t)dev_of[i] * 16];
    uint32_t c0 = ref_ab[2 * i], c1 = ref_ab[2 * i + 1];
    const float* b0 = &ref_boxes[6 * c0];
    const float* b1 = &ref_boxes[6 * c1];
    o[0] = b0[0]; o[1] = b0[1]; o[2] = b0[2]; o[3] = b0[3];
    o[4] = b0[4]; o[5] = b0[5]; o[6] = b1[0]; o[7] = b1[1];
    o[8] = b1[2]; o[9] = b1[3]; o[10] = b1[4]; o[11] = b1[5];
    int32_t r0 = (ref_ab[2 * c0] & kLeafBit) ? leaf_code(c0) : dev_of[c0];
    int32_t r1 = (ref_ab[2 * c1] & kLeafBit) ? leaf_code(c1) : dev_of[c1];
    std::memcpy(&o[12], &r0, 4);
    std::memcpy(&o[13], &r1, 4);
  }
  return 0;
}

int32_t flatten_bvh4(const std::vector<float>& ref_boxes, const std::vector<uint32_t>& ref_ab,
                     std::vector<float>& dev_nodes, uint32_t* max_stack) {
  const size_t nref = ref_ab.size() / 2;
  dev_nodes.clear();
  *max_stack = 0;
  if (nref == 0) return 0;
  auto is_leaf = [&](uint32_t i) { return (ref_ab[2 * i] & kLeafBit) != 0; };
  auto leaf_code = [&](uint32_t i) -> int32_t {
    uint32_t start = ref_ab[2 * i] & ~kLeafBit, count = ref_ab[2 * i + 1];
    return (int32_t)~((start << 3) | (count - 1));
  };
  auto area = [&](uint32_t i) {
    const float* b = &ref_boxes[6 * i];
    const double dx = (double)b[3] - b[0], dy = (double)b[4] - b[1], dz = (double)b[5] - b[2];
    return dx * dy + dy * dz + dz * dx;
  };
  if (is_leaf(0)) return leaf_code(0);
  // children of the 4-wide node grown from binary node i
  auto gather = [&](uint32_t i, uint32_t* ch) -> int {
    int n = 2;
    ch[0] = ref_ab[2 * i];
    ch[1] = ref_ab[2 * i + 1];
    while (n < 4) {
      int best = -1;
      double ba = -1.0;
      for (int k = 0; k < n; k++)
        if (!is_leaf(ch[k]) && area(ch[k]) > ba) {
          ba = area(ch[k]);
          best = k;
        }
      if (best < 0) break;
      const uint32_t c = ch[best];
      ch[best] = ref_ab[2 * c];
      ch[n++] = ref_ab[2 * c + 1];
    }
    return n;
  };
  // siblings get consecutive indices (numbered when their parent is written).
  // A walk pushes at most (internal children - 1) entries per node on its
  // path; `need` is that sum from the root, its maximum bounds the stack.
  struct Item {
    uint32_t ref2;
    int32_t slot;
    uint32_t need;
  };
  std::vector<Item> st{{0u, 0, 0u}};
  int32_t next = 1;
  dev_nodes.assign(32, 0.0f);
  while (!st.empty()) {
    const Item it = st.back();
    st.pop_back();
    uint32_t ch[4];
    const int n = gather(it.ref2, ch);
    int32_t refs[4];
    uint32_t n_int = 0;
    for (int k = 0; k < n; k++) n_int += is_leaf(ch[k]) ? 0u : 1u;
    const uint32_t need = it.need + (n_int ? n_int - 1 : 0);
    if (need > *max_stack) *max_stack = need;
    const int32_t slot = it.slot;
    for (int k = 0; k < 4; k++) {
      if (k >= n) refs[k] = kEmpty4;
      else if (is_leaf(ch[k])) refs[k] = leaf_code(ch[k]);
      else {
        refs[k] = next++;
        st.push_back({ch[k], refs[k], need});
      }
    }
    dev_nodes.resize((size_t)next * 32, 0.0f);
    float* o = &dev_nodes[(size_t)slot * 32];
    for (int k = 0; k < n; k++) {
      const float* b = &ref_boxes[6 * ch[k]];
      o[0 + k] = b[0];
      o[4 + k] = b[3];
      o[8 + k] = b[1];
      o[12 + k] = b[4];
      o[16 + k] = b[2];
      o[20 + k] = b[5];
    }
    std::memcpy(&o[24], refs, sizeof(refs));
  }
  return 0;
}

void grow_nodes_for_fma(const std::vector<float>& dev_nodes, std::vector<float>& out, float m[3], float pad) {
  const size_t n = dev_nodes.size() / 16;
  // child box c of node k: lo at 16k + 6c + {0,1,2}, hi at 16k + 6c + {3,4,5}
  float mx[3] = {0.0f, 0.0f, 0.0f};
  for (size_t k = 0; k < n; k++)
    for (int c = 0; c < 2; c++)
      for (int j = 0; j < 6; j++) {
        const float v = std::fabs(dev_nodes[16 * k + 6 * c + j]);
        if (std::isfinite(v)) mx[j % 3] = std::max(mx[j % 3], v);
      }
  for (int a = 0; a < 3; a++) m[a] = mx[a] + 1.0f;
  out = dev_nodes;
  for (size_t k = 0; k < n; k++)
    for (int c = 0; c < 2; c++)
      for (int a = 0; a < 3; a++) {
        const float grow = std::ldexp(m[a], -19) + pad;
        float& lo = out[16 * k + 6 * c + a];
        float& hi = out[16 * k + 6 * c + 3 + a];
        lo = std::nextafter(lo - grow, -INFINITY);
        hi = std::nextafter(hi + grow, INFINITY);
      }
}

void grow_ref_boxes(std::vector<float>& boxes, const float m[3], float pad) {
  for (size_t k = 0; k < boxes.size() / 6; k++)
    for (int a = 0; a < 3; a++) {
      const float grow = std::ldexp(m[a], -19) + pad;
      boxes[6 * k + a] = std::nextafter(boxes[6 * k + a] - grow, -INFINITY);
      boxes[6 * k + 3 + a] = std::nextafter(boxes[6 * k + 3 + a] + grow, INFINITY);
    }
}

float near_tie_pad(const std::vector<float>& prim_geo) {
  // 2^-17 x the longest primitive edge: Möller–Trumbore accepts barycentrics
  // down to -1e-6 (mesh.rs:446-451), i.e. hits up to about 2e-6 x the
  // edge lengths outside the triangle, beyond its exact bounding box
  double e = 0.0;
  for (size_t i = 0; i < prim_geo.size() / 9; i++) {
    const float* g = &prim_geo[9 * i];
    const double e1 = std::sqrt((double)g[3] * g[3] + (double)g[4] * g[4] + (double)g[5] * g[5]);
    const double e2 = std::sqrt((double)g[6] * g[6] + (double)g[7] * g[7] + (double)g[8] * g[8]);
    const double e3 = std::sqrt(((double)g[6] - g[3]) * ((double)g[6] - g[3]) + ((double)g[7] - g[4]) * ((double)g[7] - g[4]) +
                                ((double)g[8] - g[5]) * ((double)g[8] - g[5]));
    e = std::max(e, std::max(e1, std::max(e2, e3)));
  }
  return (float)std::ldexp(e, -17);
}

// mesh.rs:458-461 per original triangle; .w carries the material id bits.
void tri_normals(const float* pos, const uint32_t* idx, uint32_t n_tris, const uint16_t* tri_mat,
                 std::vector<float>& out) {
  out.resize((size_t)n_tris * 4);
  for (uint32_t t = 0; t < n_tris; t++) {
    F3 a{pos[3 * idx[3 * t]], pos[3 * idx[3 * t] + 1], pos[3 * idx[3 * t] + 2]};
    F3 b{pos[3 * idx[3 * t + 1]], pos[3 * idx[3 * t + 1] + 1], pos[3 * idx[3 * t + 1] + 2]};
    F3 c{pos[3 * idx[3 * t + 2]], pos[3 * idx[3 * t + 2] + 1], pos[3 * idx[3 * t + 2] + 2]};
    F3 n = normalize(cross(sub(b, a), sub(c, a)));
    out[4 * t] = n.x;
    out[4 * t + 1] = n.y;
    out[4 * t + 2] = n.z;
    uint32_t m = tri_mat[t];
    std::memcpy(&out[4 * t + 3], &m, 4);
  }
}

// tracer.rs:148-182 precomputed per material with the job's band count.
DMat make_dmat(const omg_material& m, uint32_t nb) {
  DMat d;
  std::memset(&d, 0, sizeof(d));
  float p_t = 0.0f;
  for (uint32_t b = 0; b < nb; b++) p_t = std::fmax(p_t, m.transmission[b] * m.transmission[b]);
  float p = p_t > 1e-5f ? std::fmin(std::fmax(p_t, 0.02f), 0.5f) : 0.0f;
  d.p = p;
  d.scattering = m.scattering;
  for (uint32_t b = 0; b < nb; b++) {
    float t2 = m.transmission[b] * m.transmission[b];
    d.wt[b] = p > 0.0f ? t2 / p : 0.0f;
    float keep = std::fmax(1.0f - m.absorption[b] - t2, 0.0f);
    d.wr[b] = keep / (1.0f - p);
    d.absorption[b] = m.absorption[b];
    d.t2[b] = t2;
  }
  return d;
}

}  // namespace omg
