// C entry points of the CPU oracle — TEST INFRASTRUCTURE (see omg_oracle.hpp).
// Loaded through ctypes by the test suite, the smoke check and the
// benchmark's CPU-baseline leg only.
#include "omg_oracle.hpp"

#include <thread>

using namespace orc;

namespace {

struct MeshHandle {
  int real;  // 0: float (reference semantics), 1: double (FP64 oracle)
  Mesh<float> mf;
  Mesh<double> md;
};

struct BoxC {
  float size[3];
  Material walls[6];
};

struct BoxPanelC {
  float mn[3], mx[3];
  Material m;
};

void add_trav(TraversalStats& a, const TraversalStats& b) {
  a.node_reads += b.node_reads;
  a.prim_tests += b.prim_tests;
  a.queries += b.queries;
  a.internal_visits += b.internal_visits;
  a.leaf_visits += b.leaf_visits;
  a.child_boxes += b.child_boxes;
  a.unique_nodes += b.unique_nodes;
}

// The traversal counters as 7 words: node_reads, prim_tests, queries,
// internal_visits, leaf_visits, child_boxes, unique_nodes.
void trav_out(const TraversalStats& t, uint64_t* o) {
  o[0] = t.node_reads; o[1] = t.prim_tests; o[2] = t.queries; o[3] = t.internal_visits;
  o[4] = t.leaf_visits; o[5] = t.child_boxes; o[6] = t.unique_nodes;
}

template <class R>
std::vector<BoxPanel<R>> panels_of(const BoxPanelC* p, uint32_t n) {
  std::vector<BoxPanel<R>> v(n);
  for (uint32_t i = 0; i < n; i++) {
    v[i].mn = from_f<R>(p[i].mn);
    v[i].mx = from_f<R>(p[i].mx);
    v[i].m = p[i].m;
  }
  return v;
}

// Run rays [ray_begin, ray_end) of an n_rays trace. rng_kind 0 = the
// reference's sequential xorshift64* stream (single thread), 1 = the per-ray
// PCG stream (any thread count; ranges are contiguous per thread and summed
// in order, so the result does not depend on scheduling).
template <class R, class A, class HitFn>
void run_trace(HitFn hitfn, const TraceParams& P, const float* src, const float* lis, uint32_t n_rays,
               const float* energy, int rng_kind, uint64_t seed, uint32_t ray_begin, uint32_t ray_end, int n_threads,
               double* bins_out, double* dirs_out, uint64_t* stats_out) {
  V3<R> s = from_f<R>(src), l = from_f<R>(lis);
  R per_ray = R(1) / R(n_rays);
  size_t nbin = (size_t)P.n_bins * P.n_bands, ndir = (size_t)P.n_bins * 3;
  if (rng_kind == 0) n_threads = 1;
  if (n_threads < 1) n_threads = 1;
  uint32_t total = ray_end > ray_begin ? ray_end - ray_begin : 0;
  if ((uint32_t)n_threads > total && total > 0) n_threads = (int)total;
  std::vector<std::vector<A>> tb(n_threads, std::vector<A>(nbin, A(0)));
  std::vector<std::vector<A>> td(n_threads, std::vector<A>(ndir, A(0)));
  std::vector<TraceStats> ts(n_threads);
  auto work = [&](int w) {
    uint32_t lo = ray_begin + (uint32_t)((uint64_t)total * w / n_threads);
    uint32_t hi = ray_begin + (uint32_t)((uint64_t)total * (w + 1) / n_threads);
    if (rng_kind == 0) {
      Xorshift64 g(seed);
      // advance past rays before ray_begin is not meaningful for a shared
      // stream: the sequential stream always starts at ray 0
      for (uint32_t r = lo; r < hi; r++)
        trace_ray<R, A>(hitfn, P, s, l, per_ray, energy, g, tb[w].data(), td[w].data(), &ts[w]);
    } else {
      for (uint32_t r = lo; r < hi; r++) {
        PcgRay g((uint32_t)seed, r);
        trace_ray<R, A>(hitfn, P, s, l, per_ray, energy, g, tb[w].data(), td[w].data(), &ts[w]);
      }
    }
  };
  if (n_threads == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (int w = 0; w < n_threads; w++) th.emplace_back(work, w);
    for (auto& t : th) t.join();
  }
  for (size_t i = 0; i < nbin; i++) {
    double acc = 0;
    for (int w = 0; w < n_threads; w++) acc += (double)tb[w][i];
    bins_out[i] = acc;
  }
  for (size_t i = 0; i < ndir; i++) {
    double acc = 0;
    for (int w = 0; w < n_threads; w++) acc += (double)td[w][i];
    dirs_out[i] = acc;
  }
  if (stats_out) {
    // segments, receiver hits, then the traversal counters (trav_out)
    uint64_t seg = 0, hits = 0;
    TraversalStats tr;
    for (auto& t : ts) {
      seg += t.segments;
      hits += t.receiver_hits;
      add_trav(tr, t.trav);
    }
    stats_out[0] = seg; stats_out[1] = hits;
    trav_out(tr, stats_out + 2);
  }
}

// A mesh whose raycast_hit applies the context's tie rule.
template <class R>
struct TieMesh {
  const Mesh<R>* m;
  bool tie;
  bool raycast_hit(const V3<R>& p, const V3<R>& d, GeomHit<R>* h, TraversalStats* st = nullptr,
                   uint32_t* tri = nullptr) const {
    return m->raycast_hit(p, d, h, st, tri, tie);
  }
};

}  // namespace

extern "C" {

// ------------------------------------------------------------ MeshBuilder
void* orc_mb_new() { return new MeshBuilder(); }
void orc_mb_free(void* mb) { delete (MeshBuilder*)mb; }
uint32_t orc_mb_material(void* mb, const Material* m) { return ((MeshBuilder*)mb)->material(*m); }
uint32_t orc_mb_begin_surface(void* mb) { return ((MeshBuilder*)mb)->begin_surface(); }
void orc_mb_coarse(void* mb, float e) { ((MeshBuilder*)mb)->coarse(e); }
void orc_mb_tri(void* mb, const float* a, const float* b, const float* c, uint32_t m) {
  ((MeshBuilder*)mb)->tri(a, b, c, (uint16_t)m);
}
// Bulk quads: quad i uses corners q[12*i..], material mat[i];
// begin_surface() is called new_surface[i] times first; coarse(max_edge[i])
// is applied before the quad (0 = default limit).
void orc_mb_quads(void* mbv, const float* q, const uint16_t* mat, const uint8_t* new_surface, const float* max_edge,
                  uint32_t n) {
  MeshBuilder* mb = (MeshBuilder*)mbv;
  for (uint32_t i = 0; i < n; i++) {
    if (new_surface) for (uint8_t k = 0; k < new_surface[i]; k++) mb->begin_surface();
    if (max_edge) mb->coarse(max_edge[i]);
    mb->quad(q + 12 * i, q + 12 * i + 3, q + 12 * i + 6, q + 12 * i + 9, mat[i]);
  }
}
void orc_mb_abox(void* mb, const float* mn, const float* mx, uint32_t m) { ((MeshBuilder*)mb)->abox(mn, mx, (uint16_t)m); }
void orc_mb_counts(void* mbv, uint32_t* nv, uint32_t* nt, uint32_t* nm) {
  MeshBuilder* mb = (MeshBuilder*)mbv;
  *nv = (uint32_t)(mb->positions.size() / 3);
  *nt = (uint32_t)mb->tri_material.size();
  *nm = (uint32_t)mb->materials.size();
}
void orc_mb_export(void* mbv, float* pos, uint32_t* idx, uint16_t* tri_mat, uint16_t* tri_surf, float* tri_max_edge) {
  MeshBuilder* mb = (MeshBuilder*)mbv;
  std::memcpy(pos, mb->positions.data(), mb->positions.size() * 4);
  std::memcpy(idx, mb->indices.data(), mb->indices.size() * 4);
  std::memcpy(tri_mat, mb->tri_material.data(), mb->tri_material.size() * 2);
  std::memcpy(tri_surf, mb->tri_surface.data(), mb->tri_surface.size() * 2);
  std::memcpy(tri_max_edge, mb->tri_max_edge.data(), mb->tri_max_edge.size() * 4);
}

// ------------------------------------------------------------------ Mesh
void* orc_mesh_new(int real, void* mbv) {
  MeshBuilder* mb = (MeshBuilder*)mbv;
  MeshHandle* h = new MeshHandle();
  h->real = real;
  if (real == 0) h->mf = mesh_from_builder<float>(*mb);
  else h->md = mesh_from_builder<double>(*mb);
  return h;
}
void orc_mesh_free(void* h) { delete (MeshHandle*)h; }
void orc_mesh_info(void* hv, uint32_t* n_nodes, uint32_t* n_prims, uint32_t* n_tris) {
  MeshHandle* h = (MeshHandle*)hv;
  if (h->real == 0) { *n_nodes = (uint32_t)h->mf.nodes.size(); *n_prims = (uint32_t)h->mf.packed.size(); *n_tris = (uint32_t)h->mf.tri_count(); }
  else { *n_nodes = (uint32_t)h->md.nodes.size(); *n_prims = (uint32_t)h->md.packed.size(); *n_tris = (uint32_t)h->md.tri_count(); }
}
// Flattened BVH exactly as the reference's visit_bvh sees it (mesh.rs:470-481):
// nodes as {bmin[3], a, bmax[3], b} and prims as {a[3], e1[3], e2[3], tri, material}.
// float mode only (the layout the GPU library must reproduce).
int orc_mesh_export_bvh(void* hv, float* node_boxes /*n*6*/, uint32_t* node_ab /*n*2*/, float* prim_geo /*p*9*/,
                        uint32_t* prim_tri, uint16_t* prim_mat) {
  MeshHandle* h = (MeshHandle*)hv;
  if (h->real != 0) return -1;
  const Mesh<float>& m = h->mf;
  for (size_t i = 0; i < m.nodes.size(); i++) {
    const BvhNode<float>& n = m.nodes[i];
    float* o = node_boxes + 6 * i;
    o[0] = n.bmin.x; o[1] = n.bmin.y; o[2] = n.bmin.z; o[3] = n.bmax.x; o[4] = n.bmax.y; o[5] = n.bmax.z;
    node_ab[2 * i] = n.a; node_ab[2 * i + 1] = n.b;
  }
  for (size_t i = 0; i < m.packed.size(); i++) {
    const PackedTri<float>& p = m.packed[i];
    float* o = prim_geo + 9 * i;
    o[0] = p.a.x; o[1] = p.a.y; o[2] = p.a.z; o[3] = p.e1.x; o[4] = p.e1.y; o[5] = p.e1.z;
    o[6] = p.e2.x; o[7] = p.e2.y; o[8] = p.e2.z;
    prim_tri[i] = p.tri; prim_mat[i] = p.material;
  }
  return 0;
}

// Closest hit per query (mesh.rs:484-541). flags bit 0: scan every triangle;
// bit 1: the near-tie rule (lowest surface id).
// t = -1 and tri = 0xFFFFFFFF on a miss. stats: node reads, prim tests.
int orc_mesh_raycast(void* hv, const float* o, const float* d, uint32_t n, int brute, double* t_out, uint32_t* tri_out,
                     uint64_t* stats) {
  MeshHandle* h = (MeshHandle*)hv;
  TraversalStats st;
  for (uint32_t i = 0; i < n; i++) {
    bool hit;
    double t = -1; uint32_t tri = 0xFFFFFFFFu;
    if (h->real == 0) {
      float tf; uint32_t tr;
      V3<float> oo = from_f<float>(o + 3 * i), dd = from_f<float>(d + 3 * i);
      hit = (brute & 1) ? h->mf.raycast_brute(oo, dd, &tf, &tr) : h->mf.raycast(oo, dd, &tf, &tr, &st, (brute & 2) != 0);
      if (hit) { t = tf; tri = tr; }
    } else {
      double td; uint32_t tr;
      V3<double> oo = from_f<double>(o + 3 * i), dd = from_f<double>(d + 3 * i);
      hit = (brute & 1) ? h->md.raycast_brute(oo, dd, &td, &tr) : h->md.raycast(oo, dd, &td, &tr, &st, (brute & 2) != 0);
      if (hit) { t = td; tri = tr; }
    }
    t_out[i] = t;
    tri_out[i] = tri;
  }
  if (stats) trav_out(st, stats);
  return 0;
}

// All crossings of a->b (mesh.rs:546-604). Returns the count (may exceed cap;
// only the first cap are written).
uint32_t orc_mesh_segment_hits(void* hv, const float* a, const float* b, double* t, uint32_t* tri, uint16_t* mat,
                               uint32_t cap) {
  MeshHandle* h = (MeshHandle*)hv;
  std::vector<SegHit> out;
  if (h->real == 0) h->mf.segment_hits(from_f<float>(a), from_f<float>(b), out);
  else h->md.segment_hits(from_f<double>(a), from_f<double>(b), out);
  for (size_t i = 0; i < out.size() && i < cap; i++) { t[i] = out[i].t; tri[i] = out[i].tri; mat[i] = out[i].material; }
  return (uint32_t)out.size();
}

// --------------------------------------------------------------- tracing
// tracer.rs:80-202 over the analytic shoebox (scene.rs:27-88), with optional
// panel overlays (scene.rs:90-137). Outputs double arrays: bins
// (n_bins x n_bands) and dirs (n_bins x 3). stats: segments, receiver hits,
// node reads, prim tests. rng_kind: 0 xorshift, 1 per-ray PCG; | ACC64 sums
// the f32 trajectories' contributions in double instead of f32.
constexpr int ACC64 = 0x10;
int orc_trace_box(int real, const BoxC* box, const BoxPanelC* panels, uint32_t n_panels, const TraceParams* P,
                  const float* src, const float* lis, uint32_t n_rays, const float* energy, int rng_kind,
                  uint64_t seed, uint32_t ray_begin, uint32_t ray_end, int n_threads, double* bins, double* dirs,
                  uint64_t* stats) {
  if (P->n_bands > (uint32_t)MAXB || P->n_bands == 0 || n_rays == 0) return -1;
  if (real == 0) {
    Shoebox<float> sb; sb.size = from_f<float>(box->size);
    for (int i = 0; i < 6; i++) sb.walls[i] = box->walls[i];
    auto pn = panels_of<float>(panels, n_panels);
    auto fn = [&](const V3<float>& p, const V3<float>& d, GeomHit<float>* h, uint32_t*, TraversalStats*) {
      return pn.empty() ? sb.raycast_hit(p, d, h) : with_panels_hit<float>(sb, pn, p, d, h);
    };
    if (rng_kind & ACC64)
      run_trace<float, double>(fn, *P, src, lis, n_rays, energy, rng_kind & 0xF, seed, ray_begin, ray_end, n_threads, bins, dirs, stats);
    else
      run_trace<float, float>(fn, *P, src, lis, n_rays, energy, rng_kind & 0xF, seed, ray_begin, ray_end, n_threads, bins, dirs, stats);
  } else {
    Shoebox<double> sb; sb.size = from_f<double>(box->size);
    for (int i = 0; i < 6; i++) sb.walls[i] = box->walls[i];
    auto pn = panels_of<double>(panels, n_panels);
    auto fn = [&](const V3<double>& p, const V3<double>& d, GeomHit<double>* h, uint32_t*, TraversalStats*) {
      return pn.empty() ? sb.raycast_hit(p, d, h) : with_panels_hit<double>(sb, pn, p, d, h);
    };
    run_trace<double, double>(fn, *P, src, lis, n_rays, energy, rng_kind & 0xF, seed, ray_begin, ray_end, n_threads, bins, dirs, stats);
  }
  return 0;
}

int orc_trace_mesh(int real, void* hv, const BoxPanelC* panels, uint32_t n_panels, const TraceParams* P,
                   const float* src, const float* lis, uint32_t n_rays, const float* energy, int rng_kind,
                   uint64_t seed, uint32_t ray_begin, uint32_t ray_end, int n_threads, double* bins, double* dirs,
                   uint64_t* stats) {
  MeshHandle* h = (MeshHandle*)hv;
  if (P->n_bands > (uint32_t)MAXB || P->n_bands == 0 || n_rays == 0 || h->real != real) return -1;
  if (real == 0) {
    auto pn = panels_of<float>(panels, n_panels);
    const Mesh<float>& m = h->mf;
    auto fn = [&](const V3<float>& p, const V3<float>& d, GeomHit<float>* g, uint32_t* tri, TraversalStats* st) {
      TieMesh<float> tm{&m, P->tie_mode != 0};
      if (pn.empty()) return tm.raycast_hit(p, d, g, st, tri);
      return with_panels_hit<float>(tm, pn, p, d, g, st);
    };
    if (rng_kind & ACC64)
      run_trace<float, double>(fn, *P, src, lis, n_rays, energy, rng_kind & 0xF, seed, ray_begin, ray_end, n_threads, bins, dirs, stats);
    else
      run_trace<float, float>(fn, *P, src, lis, n_rays, energy, rng_kind & 0xF, seed, ray_begin, ray_end, n_threads, bins, dirs, stats);
  } else {
    auto pn = panels_of<double>(panels, n_panels);
    const Mesh<double>& m = h->md;
    auto fn = [&](const V3<double>& p, const V3<double>& d, GeomHit<double>* g, uint32_t* tri, TraversalStats* st) {
      TieMesh<double> tm{&m, P->tie_mode != 0};
      if (pn.empty()) return tm.raycast_hit(p, d, g, st, tri);
      return with_panels_hit<double>(tm, pn, p, d, g, st);
    };
    run_trace<double, double>(fn, *P, src, lis, n_rays, energy, rng_kind & 0xF, seed, ray_begin, ray_end, n_threads, bins, dirs, stats);
  }
  return 0;
}

// Per-segment log of a mesh trace (single thread, per-ray stream): for each
// bounce-loop iteration, origin[3], dir[3] and the closest-hit ORIGINAL tri id
// (0xFFFFFFFF = miss or panel). Returns the number of segments (may exceed cap).
uint32_t orc_trace_mesh_log(int real, void* hv, const TraceParams* P, const float* src, const float* lis,
                            uint32_t n_rays, const float* energy, uint32_t seed, uint32_t ray_begin, uint32_t ray_end,
                            float* seg_out, uint32_t* tri_out, uint32_t cap) {
  MeshHandle* h = (MeshHandle*)hv;
  std::vector<uint32_t> lt;
  std::vector<float> ls;
  size_t nbin = (size_t)P->n_bins * P->n_bands;
  if (real == 0) {
    std::vector<float> bins(nbin), dirs(P->n_bins * 3);
    const Mesh<float>& m = h->mf;
    auto fn = [&](const V3<float>& p, const V3<float>& d, GeomHit<float>* g, uint32_t* tri, TraversalStats*) { return m.raycast_hit(p, d, g, nullptr, tri); };
    V3<float> s = from_f<float>(src), l = from_f<float>(lis);
    for (uint32_t r = ray_begin; r < ray_end; r++) {
      PcgRay g(seed, r);
      trace_ray<float, float>(fn, *P, s, l, 1.0f / (float)n_rays, energy, g, bins.data(), dirs.data(), nullptr, &lt, &ls);
    }
  } else {
    std::vector<double> bins(nbin), dirs(P->n_bins * 3);
    const Mesh<double>& m = h->md;
    auto fn = [&](const V3<double>& p, const V3<double>& d, GeomHit<double>* g, uint32_t* tri, TraversalStats*) { return m.raycast_hit(p, d, g, nullptr, tri); };
    V3<double> s = from_f<double>(src), l = from_f<double>(lis);
    for (uint32_t r = ray_begin; r < ray_end; r++) {
      PcgRay g(seed, r);
      trace_ray<double, double>(fn, *P, s, l, 1.0 / (double)n_rays, energy, g, bins.data(), dirs.data(), nullptr, &lt, &ls);
    }
  }
  for (size_t i = 0; i < lt.size() && i < cap; i++) {
    tri_out[i] = lt[i];
    for (int k = 0; k < 6; k++) seg_out[6 * i + k] = ls[6 * i + k];
  }
  return (uint32_t)lt.size();
}

// The same log for a trace with panels and the context's near-tie rule
// (P->tie_mode), f32 only: the segments the tracer itself walks.
uint32_t orc_trace_mesh_log_panels(void* hv, const BoxPanelC* panels, uint32_t n_panels, const TraceParams* P,
                                   const float* src, const float* lis, uint32_t n_rays, const float* energy,
                                   uint32_t seed, uint32_t ray_begin, uint32_t ray_end, float* seg_out,
                                   uint32_t* tri_out, uint32_t cap) {
  MeshHandle* h = (MeshHandle*)hv;
  if (h->real != 0) return 0;
  std::vector<uint32_t> lt;
  std::vector<float> ls;
  size_t nbin = (size_t)P->n_bins * P->n_bands;
  std::vector<float> bins(nbin), dirs(P->n_bins * 3);
  auto pn = panels_of<float>(panels, n_panels);
  const Mesh<float>& m = h->mf;
  auto fn = [&](const V3<float>& p, const V3<float>& d, GeomHit<float>* g, uint32_t* tri, TraversalStats* st) {
    TieMesh<float> tm{&m, P->tie_mode != 0};
    if (pn.empty()) return tm.raycast_hit(p, d, g, st, tri);
    return with_panels_hit<float>(tm, pn, p, d, g, st);
  };
  V3<float> s = from_f<float>(src), l = from_f<float>(lis);
  for (uint32_t r = ray_begin; r < ray_end; r++) {
    PcgRay g(seed, r);
    trace_ray<float, float>(fn, *P, s, l, 1.0f / (float)n_rays, energy, g, bins.data(), dirs.data(), nullptr, &lt,
                            &ls);
  }
  for (size_t i = 0; i < lt.size() && i < cap; i++) {
    tri_out[i] = lt[i];
    for (int k = 0; k < 6; k++) seg_out[6 * i + k] = ls[6 * i + k];
  }
  return (uint32_t)lt.size();
}

// ---------------------------------------------------------------- reverb
// tracer.rs:204-257. level_f32 != 0 sums the late energy in f32 as the
// reference does; 0 sums it in double (FP64 oracle).
void orc_estimate_reverb(const double* bins, uint32_t n_bins, uint32_t nb, float bin_dt, int level_f32, float* rt60,
                         float* level, double* rt60_fit) {
  if (level_f32) {
    std::vector<float> bf(bins, bins + (size_t)n_bins * nb);
    estimate_reverb<float, float>(bf.data(), n_bins, nb, bin_dt, rt60, level, rt60_fit);
  } else {
    estimate_reverb<double, double>(bins, n_bins, nb, bin_dt, rt60, level, rt60_fit);
  }
}

// tracer.rs:62-77
void orc_late_direction(const double* bins, const double* dirs, uint32_t n_bins, uint32_t nb, uint32_t mid,
                        float bin_dt, float from_s, int f32, float* dir, float* aniso) {
  if (f32) {
    std::vector<float> bf(bins, bins + (size_t)n_bins * nb), df(dirs, dirs + (size_t)n_bins * 3);
    late_direction<float>(bf.data(), df.data(), n_bins, nb, mid, bin_dt, from_s, dir, aniso);
  } else {
    late_direction<double>(bins, dirs, n_bins, nb, mid, bin_dt, from_s, dir, aniso);
  }
}

// ------------------------------------------------------------------ dome
struct DomeHandle {
  MeshHandle* mesh;
  std::vector<DomePanel> glass;
  std::vector<V3<float>> fan_f;
  std::vector<V3<double>> fan_d;
  std::vector<float> ema;
  int primed = 0;
  bool tie = false;
};

void* orc_dome_new(void* meshv, const DomePanel* glass, uint32_t n_glass, uint32_t n_fan, uint32_t nb, int tie) {
  DomeHandle* d = new DomeHandle();
  d->tie = tie != 0;
  d->mesh = (MeshHandle*)meshv;
  d->glass.assign(glass, glass + n_glass);
  if (d->mesh->real == 0) d->fan_f = dome_fan<float>(n_fan);
  else d->fan_d = dome_fan<double>(n_fan);
  d->ema.assign(9 * nb, 0.0f);
  return d;
}
void orc_dome_free(void* d) { delete (DomeHandle*)d; }

// dome.rs:424-478. stats: escape events, through calls, node reads, prim tests.
int orc_dome_sample(void* dv, const float* eye, const DomePanel* leaves, uint32_t n_leaves, uint32_t n_rays,
                    uint32_t max_events, uint32_t nb, float ema_alpha, float* out_dir, float* out_energy,
                    double* raw_energy, uint8_t* escape_flags, float* ray_tp, uint64_t* stats) {
  DomeHandle* d = (DomeHandle*)dv;
  if (nb > (uint32_t)MAXB || nb < 2 || d->ema.size() != 9 * nb || n_rays == 0) return -1;
  std::vector<DomePanel> lv(leaves, leaves + n_leaves);
  DomeStats st;
  if (d->mesh->real == 0) {
    if (n_rays > d->fan_f.size()) return -1;
    dome_sample<float>(d->mesh->mf, d->glass, lv, d->fan_f, from_f<float>(eye), n_rays, max_events, nb, ema_alpha,
                       d->ema.data(), &d->primed, out_dir, out_energy, raw_energy, escape_flags, ray_tp, &st, d->tie);
  } else {
    if (n_rays > d->fan_d.size()) return -1;
    dome_sample<double>(d->mesh->md, d->glass, lv, d->fan_d, from_f<double>(eye), n_rays, max_events, nb, ema_alpha,
                        d->ema.data(), &d->primed, out_dir, out_energy, raw_energy, escape_flags, ray_tp, &st, d->tie);
  }
  if (stats) {
    stats[0] = st.escape_events; stats[1] = st.through_calls;
    trav_out(st.trav, stats + 2);
  }
  return 0;
}

// dome.rs:313-324 fan directions (for the GPU dome test).
void orc_dome_fan(uint32_t n, int real, double* out) {
  if (real == 0) { auto f = dome_fan<float>(n); for (uint32_t i = 0; i < n; i++) { out[3*i] = f[i].x; out[3*i+1] = f[i].y; out[3*i+2] = f[i].z; } }
  else { auto f = dome_fan<double>(n); for (uint32_t i = 0; i < n; i++) { out[3*i] = f[i].x; out[3*i+1] = f[i].y; out[3*i+2] = f[i].z; } }
}

// Per-ray stream probe: the first n draws of ray `ray` (for the RNG test).
void orc_pcg_draws(uint32_t seed, uint32_t ray, uint32_t n, uint32_t* out) {
  PcgRay g(seed, ray);
  for (uint32_t i = 0; i < n; i++) out[i] = g.next_u32();
}
void orc_xorshift_draws(uint64_t seed, uint32_t n, uint64_t* out) {
  Xorshift64 g(seed);
  for (uint32_t i = 0; i < n; i++) out[i] = g.next_u64();
}

int orc_abi_version() { return 1; }
}

extern "C" {
// dome.rs:121-258 into an oracle MeshBuilder; writes up to glass_cap panes.
// Returns the pane count. wall_max_edge = 0 keeps the reference's default limit.
uint32_t orc_world_build(void* mbv, const RoomC* rooms, uint32_t n_rooms, const DoorC* doors, uint32_t n_doors,
                         float town0, float town1, float wall_max_edge, uint32_t nb, DomePanel* glass,
                         uint32_t glass_cap) {
  std::vector<RoomC> r(rooms, rooms + n_rooms);
  std::vector<DoorC> d(doors, doors + n_doors);
  auto g = build_world_mesh(*(MeshBuilder*)mbv, r, d, town0, town1, wall_max_edge, (int)nb);
  for (size_t i = 0; i < g.size() && i < glass_cap; i++) glass[i] = g[i];
  return (uint32_t)g.size();
}
}

extern "C" void orc_sincos_f32(const float* phi, uint32_t n, float* s, float* c) {
  for (uint32_t i = 0; i < n; i++) sincos_f32(phi[i], &s[i], &c[i]);
}

// ------------------------------------------------ world early reflections
// crates/omg-core/src/pt_mesh.rs over an f32 oracle mesh (omg_oracle_early.hpp).
#include "omg_oracle_early.hpp"

namespace {
struct EarlyHandle {
  const Mesh<float>* mesh;
  SurfaceTable table;
  std::vector<std::pair<V3<float>, V3<float>>> boxes;
};
}  // namespace

extern "C" {
// SurfaceTable::build + append_box per furniture box (early_world.rs:114-120);
// the boxes are also discovery's overlay reflectors.
void* orc_early_new(void* meshv, const BoxPanelC* furn, uint32_t n_furn) {
  MeshHandle* h = (MeshHandle*)meshv;
  if (h->real != 0) return nullptr;
  EarlyHandle* e = new EarlyHandle();
  e->mesh = &h->mf;
  e->table.build(h->mf);
  for (uint32_t i = 0; i < n_furn; i++) {
    e->table.append_box(furn[i].mn, furn[i].mx, furn[i].m);
    e->boxes.push_back({from_f<float>(furn[i].mn), from_f<float>(furn[i].mx)});
  }
  return e;
}
void orc_early_free(void* e) { delete (EarlyHandle*)e; }
uint32_t orc_early_base_overlay(void* e) { return ((EarlyHandle*)e)->table.base_overlay; }
uint32_t orc_early_n_surfaces(void* e) { return (uint32_t)((EarlyHandle*)e)->table.surfaces.size(); }

// mesh_chains (pt_mesh.rs:382-457); use_boxes = 0 runs it with no overlay
// boxes (the furniture switch off). Returns the chain count; writes <= cap.
uint32_t orc_early_discover(void* ev, const float* lis, uint32_t n_rays, uint32_t rot, int use_boxes,
                            uint16_t* chains, uint8_t* orders, uint32_t cap) {
  EarlyHandle* e = (EarlyHandle*)ev;
  std::vector<MChain> out;
  static const std::vector<std::pair<V3<float>, V3<float>>> none;
  mesh_chains(*e->mesh, use_boxes ? e->boxes : none, e->table.base_overlay, from_f<float>(lis), n_rays, rot, out);
  for (size_t i = 0; i < out.size() && i < cap; i++) {
    for (int k = 0; k < M_MAX_ORDER; k++) chains[3 * i + k] = out[i].c[k];
    orders[i] = out[i].order;
  }
  return (uint32_t)out.size();
}

// mesh_record (pt_mesh.rs:186-337) for every (source, chain) pair, source
// major; out: 7 floats per pair (delay_s, dir[3], gains[3]), valid: 1 when the
// pair solves. threads > 1 splits the sources over std::threads.
void orc_early_solve(void* ev, const uint16_t* src_ids, const float* src_pos, uint32_t n_src, const uint16_t* chains,
                     const uint8_t* orders, uint32_t n_chains, const float* lis, const Aabb* extras, uint32_t n_extras,
                     float* out, uint8_t* valid, int threads) {
  EarlyHandle* e = (EarlyHandle*)ev;
  std::vector<Aabb> ex(extras, extras + n_extras);
  const V3<float> L = from_f<float>(lis);
  auto run = [&](uint32_t s0, uint32_t s1) {
    std::vector<SegHit> buf;
    for (uint32_t s = s0; s < s1; s++) {
      for (uint32_t c = 0; c < n_chains; c++) {
        MeshRecord r;
        const size_t k = (size_t)s * n_chains + c;
        const bool ok = mesh_record(*e->mesh, e->table, chains + 3 * c, orders[c], src_ids[s],
                                    from_f<float>(src_pos + 3 * s), L, ex, buf, &r);
        valid[k] = ok ? 1 : 0;
        float* o = out + 7 * k;
        if (ok) {
          o[0] = r.delay_s;
          for (int q = 0; q < 3; q++) { o[1 + q] = r.dir[q]; o[4 + q] = r.gains[q]; }
        } else {
          for (int q = 0; q < 7; q++) o[q] = 0.0f;
        }
      }
    }
  };
  const uint32_t nt = (uint32_t)std::max(1, std::min<int>(threads, (int)std::max<uint32_t>(n_src, 1)));
  if (nt <= 1) {
    run(0, n_src);
    return;
  }
  std::vector<std::thread> ts;
  for (uint32_t t = 0; t < nt; t++) ts.emplace_back(run, n_src * t / nt, n_src * (t + 1) / nt);
  for (auto& t : ts) t.join();
}
}
