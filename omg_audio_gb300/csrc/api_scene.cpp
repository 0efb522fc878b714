// C ABI of the GB300 tracer (include/omg_cuda.h), part 2: mesh builder,
// scene upload (reference SAH tree on the host or LBVH on the device), BVH
// export, closest-hit queries, estimate_reverb.
#include <limits>

#include "runtime.h"

using namespace omg;

struct omg_mesh_builder {
  MeshBuilder mb;
};

namespace {

// Device-side arrays of a scene from its tessellated primitives.
int32_t upload_scene_arrays(omg_ctx* ctx, SceneRec& S, const std::vector<float>& prim_geo,
                            const std::vector<uint32_t>& prim_tri, const std::vector<uint16_t>& prim_mat,
                            const std::vector<uint16_t>& prim_surf, const std::vector<float>& normals,
                            const std::vector<DMat>& dmats, const std::vector<uint16_t>& tri_surface) {
  size_t np = prim_tri.size();
  std::vector<float> pr(np * 12, 0.0f);
  for (size_t i = 0; i < np; i++) {
    const float* g = &prim_geo[9 * i];
    float* o = &pr[12 * i];
    o[0] = g[0]; o[1] = g[1]; o[2] = g[2];
    uint32_t m = prim_mat[i], t = prim_tri[i], s = prim_surf.empty() ? 0u : prim_surf[i];
    std::memcpy(&o[3], &m, 4);
    o[4] = g[3]; o[5] = g[4]; o[6] = g[5];
    std::memcpy(&o[7], &t, 4);
    o[8] = g[6]; o[9] = g[7]; o[10] = g[8];
    std::memcpy(&o[11], &s, 4);
  }
  CK(S.prims.alloc(np * 3));
  if (np) CK(cudaMemcpy(S.prims.p, pr.data(), pr.size() * 4, cudaMemcpyHostToDevice));
  CK(S.normals.alloc(normals.size() / 4));
  if (!normals.empty()) CK(cudaMemcpy(S.normals.p, normals.data(), normals.size() * 4, cudaMemcpyHostToDevice));
  CK(S.mats.alloc(dmats.size()));
  if (!dmats.empty()) CK(cudaMemcpy(S.mats.p, dmats.data(), dmats.size() * sizeof(DMat), cudaMemcpyHostToDevice));
  CK(S.tri_surface.alloc(tri_surface.size()));
  if (!tri_surface.empty())
    CK(cudaMemcpy(S.tri_surface.p, tri_surface.data(), tri_surface.size() * 2, cudaMemcpyHostToDevice));
  return OMG_OK;
}

// The exact vertices of every primitive in leaf order (watertight contexts):
// A, B, C in .xyz with the primitive's own .w words (material, triangle,
// surface), so a walk reads its ids from either array. vtx: 9 floats per
// primitive in tessellation order; perm: tessellation index per position.
int32_t upload_exact_vertices(omg_ctx* ctx, SceneRec& S, const std::vector<float>& vtx,
                              const std::vector<uint32_t>& perm, const std::vector<uint16_t>& psurf) {
  const size_t np = S.prim_tri.size();
  if (np == 0) return OMG_OK;
  if (perm.size() != np || vtx.size() != 9 * np) return OMG_E_INVALID;
  std::vector<float> pr(np * 12);
  for (size_t i = 0; i < np; i++) {
    const float* v = &vtx[9 * (size_t)perm[i]];
    float* o = &pr[12 * i];
    const uint32_t m = S.prim_mat[i], t = S.prim_tri[i], s = psurf.empty() ? 0u : psurf[i];
    o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; std::memcpy(&o[3], &m, 4);
    o[4] = v[3]; o[5] = v[4]; o[6] = v[5]; std::memcpy(&o[7], &t, 4);
    o[8] = v[6]; o[9] = v[7]; o[10] = v[8]; std::memcpy(&o[11], &s, 4);
  }
  CK(S.prims_wt.alloc(np * 3));
  CK(cudaMemcpy(S.prims_wt.p, pr.data(), pr.size() * 4, cudaMemcpyHostToDevice));
  return OMG_OK;
}

// The three-axis tree built on the GPU (sah3.cu): the tessellated primitives
// go up in tessellation order, the tree comes back in build_sah3's form, and
// the host's primitive arrays are put in its leaf order.
int32_t build_sah3_on_device(omg_ctx* ctx, SceneRec& S, std::vector<uint32_t>* perm_out) {
  const size_t np = S.prim_tri.size();
  if (np == 0) {
    S.ref_boxes.clear();
    S.ref_ab.clear();
    return OMG_OK;
  }
  std::vector<float> pr(np * 12, 0.0f);
  for (size_t i = 0; i < np; i++) {
    const float* g = &S.prim_geo[9 * i];
    float* o = &pr[12 * i];
    o[0] = g[0]; o[1] = g[1]; o[2] = g[2];
    o[4] = g[3]; o[5] = g[4]; o[6] = g[5];
    o[8] = g[6]; o[9] = g[7]; o[10] = g[8];
  }
  DevBuf<float4> d;
  CK(d.alloc(np * 3));
  CK(cudaMemcpy(d.p, pr.data(), pr.size() * 4, cudaMemcpyHostToDevice));
  std::vector<uint32_t> perm;
  CK(sah3_build_device(d.p, (uint32_t)np, S.ref_boxes, S.ref_ab, perm, ctx->stream));
  std::vector<float> geo(S.prim_geo.size());
  std::vector<uint32_t> tri(np);
  std::vector<uint16_t> mat(np);
  for (size_t i = 0; i < np; i++) {
    const uint32_t j = perm[i];
    if (j >= np) return OMG_E_INVALID;
    std::memcpy(&geo[9 * i], &S.prim_geo[9 * (size_t)j], 9 * sizeof(float));
    tri[i] = S.prim_tri[j];
    mat[i] = S.prim_mat[j];
  }
  S.prim_geo.swap(geo);
  S.prim_tri.swap(tri);
  S.prim_mat.swap(mat);
  if (perm_out) perm_out->swap(perm);
  return OMG_OK;
}

int32_t scene_upload_impl(omg_ctx* ctx, const float* pos, uint32_t nv, const uint32_t* idx, uint32_t nt,
                          const uint16_t* tri_mat, const float* tri_max_edge, const uint16_t* tri_surf,
                          const omg_material* mats, uint32_t nm, uint32_t nb, uint32_t kind, uint32_t* scene_id) {
  if (!ctx || !scene_id || nb == 0 || nb > (uint32_t)MAXB || (nt && (!pos || !idx || !tri_mat)) || (nm && !mats) ||
      (kind != OMG_BVH_SAH && kind != OMG_BVH_LBVH && kind != OMG_BVH_SAH3 && kind != OMG_BVH_SAH3_HOST))
    return OMG_E_INVALID;
  for (uint32_t t = 0; t < nt; t++) {
    if (tri_mat[t] >= nm) return OMG_E_INVALID;
    for (int k = 0; k < 3; k++)
      if (idx[3 * t + k] >= nv) return OMG_E_INVALID;
  }
  for (uint32_t v = 0; v < 3 * nv; v++)
    if (!std::isfinite(pos[v])) return OMG_E_INVALID;
  for (uint32_t m = 0; m < nm; m++)
    if (!valid_material(mats[m], nb)) return OMG_E_INVALID;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, cudaGetLastError(), "cudaSetDevice");

  std::unique_ptr<SceneRec> S(new SceneRec());
  S->n_tris = nt;
  S->n_bands = nb;
  S->bvh_kind = kind;
  // watertight contexts keep every primitive's exact vertices (prims_wt)
  const bool wt = ctx->prm.tri_test == OMG_TRI_WATERTIGHT;
  std::vector<float> vtx;
  std::vector<uint32_t> perm;
  tessellate(pos, idx, nt, tri_mat, tri_max_edge, S->prim_geo, S->prim_tri, S->prim_mat, wt ? &vtx : nullptr);
  S->n_prims = (uint32_t)S->prim_tri.size();
  if (S->n_prims >= (1u << 28)) return OMG_E_INVALID;
  std::vector<float> normals;
  tri_normals(pos, idx, nt, tri_mat, normals);
  std::vector<DMat> dmats(nm);
  for (uint32_t m = 0; m < nm; m++) dmats[m] = make_dmat(mats[m], nb);
  std::vector<uint16_t> tsurf(nt, 0);
  if (tri_surf) tsurf.assign(tri_surf, tri_surf + nt);
  // the surface table's seed (SurfaceTable::build, pt_mesh.rs:51-78): the
  // first triangle of each surface id gives its plane and material
  S->materials.assign(mats, mats + nm);
  for (uint32_t t = 0; t < nt; t++) {
    const uint32_t sid = tsurf[t];
    if (sid >= S->surf_seed.size()) {
      SceneRec::SurfSeed blank{{0.0f, 0.0f, 1.0f}, std::numeric_limits<float>::max(), 0u, 0u};
      S->surf_seed.resize(sid + 1, blank);
    }
    SceneRec::SurfSeed& q = S->surf_seed[sid];
    if (!q.set) {
      const float* n = &normals[4 * (size_t)t];
      const float* p = &pos[3 * (size_t)idx[3 * t]];
      q.n[0] = n[0];
      q.n[1] = n[1];
      q.n[2] = n[2];
      q.d = n[0] * p[0] + n[1] * p[1] + n[2] * p[2];
      q.mat = tri_mat[t];
      q.set = 1u;
    }
  }

  if (kind == OMG_BVH_SAH || kind == OMG_BVH_SAH3 || kind == OMG_BVH_SAH3_HOST) {
    if (kind == OMG_BVH_SAH) {
      build_sah(S->prim_geo, S->prim_tri, S->prim_mat, S->ref_boxes, S->ref_ab, wt ? &perm : nullptr);
    } else if (kind == OMG_BVH_SAH3_HOST) {
      build_sah3(S->prim_geo, S->prim_tri, S->prim_mat, S->ref_boxes, S->ref_ab, wt ? &perm : nullptr);
    } else {
      int32_t rc = build_sah3_on_device(ctx, *S, wt ? &perm : nullptr);
      if (rc) return rc;
    }
    std::vector<float> dev_nodes;
    S->root = flatten_bvh2(S->ref_boxes, S->ref_ab, dev_nodes);
    S->n_nodes = (uint32_t)(dev_nodes.size() / 16);
    std::vector<uint16_t> psurf(S->n_prims);
    for (uint32_t i = 0; i < S->n_prims; i++) psurf[i] = tsurf[S->prim_tri[i]];
    int32_t rc = upload_scene_arrays(ctx, *S, S->prim_geo, S->prim_tri, S->prim_mat, psurf, normals, dmats, tsurf);
    if (rc) return rc;
    if (wt && (rc = upload_exact_vertices(ctx, *S, vtx, perm, psurf))) return rc;
    CK(S->nodes.alloc(S->n_nodes * 4));
    if (S->n_nodes)
      CK(cudaMemcpy(S->nodes.p, dev_nodes.data(), dev_nodes.size() * 4, cudaMemcpyHostToDevice));
    const float pad = near_tie_pad(S->prim_geo);
    if (S->n_nodes) {
      std::vector<float> grown;
      grow_nodes_for_fma(dev_nodes, grown, S->fast_m, pad);
      CK(S->nodes_f.alloc(S->n_nodes * 4));
      CK(cudaMemcpy(S->nodes_f.p, grown.data(), grown.size() * 4, cudaMemcpyHostToDevice));
    }
    // the 4-wide tree serves near-tie walks only: its boxes are grown likewise
    std::vector<float> grown_ref = S->ref_boxes;
    grow_ref_boxes(grown_ref, S->fast_m, pad);
    std::vector<float> dev_nodes4;
    uint32_t need = 0;
    S->root4 = flatten_bvh4(grown_ref, S->ref_ab, dev_nodes4, &need);
    S->n_nodes4 = (uint32_t)(dev_nodes4.size() / 32);
    // a tree whose walks could overflow the traversal stack keeps the binary walk
    if (need >= (uint32_t)STACK_DEPTH) S->n_nodes4 = 0;
    if (S->n_nodes4) {
      CK(S->nodes4.alloc((size_t)S->n_nodes4 * 8));
      CK(cudaMemcpy(S->nodes4.p, dev_nodes4.data(), dev_nodes4.size() * 4, cudaMemcpyHostToDevice));
      // child by child: (lo.x, lo.y, lo.z, hi.x), (hi.y, hi.z, ref, 0)
      std::vector<float> aos((size_t)S->n_nodes4 * 32, 0.0f);
      for (size_t n = 0; n < S->n_nodes4; n++) {
        const float* q = &dev_nodes4[32 * n];
        for (int k = 0; k < 4; k++) {
          float* o = &aos[32 * n + 8 * k];
          o[0] = q[0 + k];   // lo.x
          o[1] = q[8 + k];   // lo.y
          o[2] = q[16 + k];  // lo.z
          o[3] = q[4 + k];   // hi.x
          o[4] = q[12 + k];  // hi.y
          o[5] = q[20 + k];  // hi.z
          o[6] = q[24 + k];  // ref bits
        }
      }
      CK(S->nodes4c.alloc((size_t)S->n_nodes4 * 8));
      CK(cudaMemcpy(S->nodes4c.p, aos.data(), aos.size() * 4, cudaMemcpyHostToDevice));
    }
  } else {
    // LBVH: upload the primitives in tessellation order, build on the device
    std::vector<uint16_t> psurf(S->n_prims);
    for (uint32_t i = 0; i < S->n_prims; i++) psurf[i] = tsurf[S->prim_tri[i]];
    int32_t rc = upload_scene_arrays(ctx, *S, S->prim_geo, S->prim_tri, S->prim_mat, psurf, normals, dmats, tsurf);
    if (rc) return rc;
    if (S->n_prims > 0) {
      DevBuf<float4> sorted;
      CK(sorted.alloc((size_t)S->n_prims * 3));
      S->n_nodes = S->n_prims > 1 ? S->n_prims - 1 : 0;
      CK(S->nodes.alloc((size_t)std::max<uint32_t>(S->n_nodes, 1) * 4));
      DevBuf<unsigned char> scratch;
      size_t sb = lbvh_scratch_bytes(S->n_prims);
      CK(scratch.alloc(sb));
      DevBuf<int32_t> d_root;
      CK(d_root.alloc(1));
      CK(lbvh_build(S->prims.p, S->n_prims, sorted.p, S->nodes.p, d_root.p, scratch.p, sb, ctx->stream));
      CK(cudaMemcpyAsync(&S->root, d_root.p, 4, cudaMemcpyDeviceToHost, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
      std::swap(S->prims.p, sorted.p);
      std::swap(S->prims.n, sorted.n);
      if (wt) {
        // the leaf order: the sorted keys' low words (lbvh.cu keeps them past
        // its 64-byte bounds block)
        std::vector<unsigned long long> keys(S->n_prims);
        CK(cudaMemcpy(keys.data(), scratch.p + 64, keys.size() * 8, cudaMemcpyDeviceToHost));
        perm.resize(S->n_prims);
        for (uint32_t i = 0; i < S->n_prims; i++) perm[i] = (uint32_t)(keys[i] & 0xFFFFFFFFull);
      }
      // host copy of the leaf-ordered primitives for export
      std::vector<float> pr((size_t)S->n_prims * 12);
      CK(cudaMemcpy(pr.data(), S->prims.p, pr.size() * 4, cudaMemcpyDeviceToHost));
      for (uint32_t i = 0; i < S->n_prims; i++) {
        const float* o = &pr[12 * i];
        float g[9] = {o[0], o[1], o[2], o[4], o[5], o[6], o[8], o[9], o[10]};
        std::memcpy(&S->prim_geo[9 * i], g, sizeof(g));
        uint32_t m, t;
        std::memcpy(&m, &o[3], 4);
        std::memcpy(&t, &o[7], 4);
        S->prim_mat[i] = (uint16_t)m;
        S->prim_tri[i] = t;
      }
      if (wt) {
        for (uint32_t i = 0; i < S->n_prims; i++) psurf[i] = tsurf[S->prim_tri[i]];
        if ((rc = upload_exact_vertices(ctx, *S, vtx, perm, psurf))) return rc;
      }
      // grown boxes for the near-tie walks: the bound from the primitives
      float mx[3] = {0.0f, 0.0f, 0.0f};
      for (uint32_t i = 0; i < S->n_prims; i++) {
        const float* g = &S->prim_geo[9 * i];
        for (int a = 0; a < 3; a++) {
          const float p0 = g[a], p1 = g[a] + g[3 + a], p2 = g[a] + g[6 + a];
          mx[a] = std::max(mx[a], std::max(std::fabs(p0), std::max(std::fabs(p1), std::fabs(p2))));
        }
      }
      for (int a = 0; a < 3; a++) S->fast_m[a] = mx[a] + 1.0f;
      if (S->root >= 0 && S->n_nodes) {
        CK(S->nodes_f.alloc((size_t)S->n_nodes * 4));
        CK(grow_nodes(S->nodes.p, S->nodes_f.p, S->n_nodes, S->fast_m, near_tie_pad(S->prim_geo), ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
      }
    }
  }
  uint32_t id = 1;  // lowest free slot of the fixed table
  while (id < kMaxScenes && ctx->scenes.count(id)) id++;
  if (id >= kMaxScenes) return OMG_E_INVALID;
  ctx->scenes[id] = std::move(S);
  int32_t rc = sync_scene_table(ctx);
  if (rc) {
    ctx->scenes.erase(id);
    return rc;
  }
  *scene_id = id;
  return OMG_OK;
}

}  // namespace

extern "C" {

// ------------------------------------------------------------ mesh builder
omg_mesh_builder* omg_mb_create(void) { return new omg_mesh_builder(); }
void omg_mb_destroy(omg_mesh_builder* mb) { delete mb; }
uint32_t omg_mb_material(omg_mesh_builder* mb, const omg_material* m) { return mb->mb.material(*m); }
uint32_t omg_mb_begin_surface(omg_mesh_builder* mb) { return mb->mb.begin_surface(); }
void omg_mb_coarse(omg_mesh_builder* mb, float e) { mb->mb.coarse(e); }
void omg_mb_tri(omg_mesh_builder* mb, const float a[3], const float b[3], const float c[3], uint32_t m) {
  mb->mb.tri(a, b, c, m);
}
void omg_mb_quad(omg_mesh_builder* mb, const float a[3], const float b[3], const float c[3], const float d[3],
                 uint32_t m) {
  mb->mb.quad(a, b, c, d, m);
}
void omg_mb_abox(omg_mesh_builder* mb, const float mn[3], const float mx[3], uint32_t m) { mb->mb.abox(mn, mx, m); }
void omg_mb_quads(omg_mesh_builder* mb, const float* q, const uint16_t* mat, const uint8_t* ns, const float* me,
                  uint32_t n) {
  for (uint32_t i = 0; i < n; i++) {
    if (ns) for (uint8_t k = 0; k < ns[i]; k++) mb->mb.begin_surface();
    if (me) mb->mb.coarse(me[i]);
    mb->mb.quad(q + 12 * i, q + 12 * i + 3, q + 12 * i + 6, q + 12 * i + 9, mat ? mat[i] : 0);
  }
}
void omg_mb_counts(const omg_mesh_builder* mb, uint32_t* nv, uint32_t* nt, uint32_t* nm) {
  if (nv) *nv = (uint32_t)(mb->mb.positions.size() / 3);
  if (nt) *nt = (uint32_t)mb->mb.tri_material.size();
  if (nm) *nm = (uint32_t)mb->mb.materials.size();
}
void omg_mb_export(const omg_mesh_builder* mb, float* pos, uint32_t* idx, uint16_t* tm, uint16_t* ts, float* te) {
  const MeshBuilder& b = mb->mb;
  if (pos) std::memcpy(pos, b.positions.data(), b.positions.size() * 4);
  if (idx) std::memcpy(idx, b.indices.data(), b.indices.size() * 4);
  if (tm) std::memcpy(tm, b.tri_material.data(), b.tri_material.size() * 2);
  if (ts) std::memcpy(ts, b.tri_surface.data(), b.tri_surface.size() * 2);
  if (te) std::memcpy(te, b.tri_max_edge.data(), b.tri_max_edge.size() * 4);
}

// ------------------------------------------------------------------ scenes
int32_t omg_scene_upload(omg_ctx* ctx, const float* pos, uint32_t nv, const uint32_t* idx, uint32_t nt,
                         const uint16_t* tri_mat, const float* tri_max_edge, const omg_material* mats, uint32_t nm,
                         uint32_t nb, uint32_t kind, uint32_t* scene_id) {
  return scene_upload_impl(ctx, pos, nv, idx, nt, tri_mat, tri_max_edge, nullptr, mats, nm, nb, kind, scene_id);
}

int32_t omg_scene_from_builder(omg_ctx* ctx, const omg_mesh_builder* mb, uint32_t nb, uint32_t kind,
                               uint32_t* scene_id) {
  if (!mb) return OMG_E_INVALID;
  const MeshBuilder& b = mb->mb;
  return scene_upload_impl(ctx, b.positions.data(), (uint32_t)(b.positions.size() / 3), b.indices.data(),
                           (uint32_t)b.tri_material.size(), b.tri_material.data(), b.tri_max_edge.data(),
                           b.tri_surface.data(), b.materials.data(), (uint32_t)b.materials.size(), nb, kind,
                           scene_id);
}

int32_t omg_scene_release(omg_ctx* ctx, uint32_t id) {
  if (!ctx) return OMG_E_INVALID;
  auto it = ctx->scenes.find(id);
  if (it == ctx->scenes.end()) return OMG_E_NOT_FOUND;
  cudaStreamSynchronize(ctx->stream);
  ctx->scenes.erase(it);
  return sync_scene_table(ctx);
}

int32_t omg_scene_info(omg_ctx* ctx, uint32_t id, uint32_t* n_nodes, uint32_t* n_prims, uint32_t* n_tris) {
  if (!ctx) return OMG_E_INVALID;
  auto it = ctx->scenes.find(id);
  if (it == ctx->scenes.end()) return OMG_E_NOT_FOUND;
  const SceneRec& S = *it->second;
  // reference-form node count for host-built trees (leaves included), device node count otherwise
  if (n_nodes) *n_nodes = S.bvh_kind != OMG_BVH_LBVH ? (uint32_t)(S.ref_ab.size() / 2) : S.n_nodes;
  if (n_prims) *n_prims = S.n_prims;
  if (n_tris) *n_tris = S.n_tris;
  return OMG_OK;
}

int32_t omg_scene_export_bvh(omg_ctx* ctx, uint32_t id, float* node_boxes, uint32_t* node_ab, float* prim_geo,
                             uint32_t* prim_tri, uint16_t* prim_mat) {
  if (!ctx) return OMG_E_INVALID;
  auto it = ctx->scenes.find(id);
  if (it == ctx->scenes.end()) return OMG_E_NOT_FOUND;
  const SceneRec& S = *it->second;
  if (S.bvh_kind != OMG_BVH_LBVH) {
    if (node_boxes) std::memcpy(node_boxes, S.ref_boxes.data(), S.ref_boxes.size() * 4);
    if (node_ab) std::memcpy(node_ab, S.ref_ab.data(), S.ref_ab.size() * 4);
  } else if (node_boxes || node_ab) {
    return OMG_E_INVALID;  // LBVH trees have no reference-form node array
  }
  if (prim_geo) std::memcpy(prim_geo, S.prim_geo.data(), S.prim_geo.size() * 4);
  if (prim_tri) std::memcpy(prim_tri, S.prim_tri.data(), S.prim_tri.size() * 4);
  if (prim_mat) std::memcpy(prim_mat, S.prim_mat.data(), S.prim_mat.size() * 2);
  return OMG_OK;
}

// ----------------------------------------------------------- mesh queries
int32_t omg_raycast(omg_ctx* ctx, uint32_t id, const float* o, const float* d, uint32_t n, float* t, uint32_t* tri) {
  if (!ctx || (n && (!o || !d || !t || !tri))) return OMG_E_INVALID;
  if (ctx->scenes.find(id) == ctx->scenes.end()) return OMG_E_NOT_FOUND;
  if (n == 0) return OMG_OK;
  if (ctx->q_o.n < 3ull * n) {
    CK(ctx->q_o.alloc(3ull * n));
    CK(ctx->q_d.alloc(3ull * n));
    CK(ctx->q_t.alloc(n));
    CK(ctx->q_tri.alloc(n));
  }
  if (!ctx->q_hdr.p) CK(ctx->q_hdr.alloc(1));
  cudaStream_t s = ctx->stream;
  CK(cudaMemsetAsync(ctx->q_hdr.p, 0, sizeof(DLaunch), s));
  CK(cudaMemcpyAsync(ctx->q_o.p, o, 12ull * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->q_d.p, d, 12ull * n, cudaMemcpyHostToDevice, s));
  CK(launch_raycast(ctx->d_scenes.p + id, ctx->q_o.p, ctx->q_d.p, n, ctx->q_t.p, ctx->q_tri.p, ctx->q_hdr.p,
                    ctx->prm.tie_mode != 0, s));
  CK(cudaMemcpyAsync(t, ctx->q_t.p, 4ull * n, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(tri, ctx->q_tri.p, 4ull * n, cudaMemcpyDeviceToHost, s));
  DLaunch h;
  CK(cudaMemcpyAsync(&h, ctx->q_hdr.p, sizeof(DLaunch), cudaMemcpyDeviceToHost, s));
  cudaEvent_t ev;
  CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  CK(cudaEventRecord(ev, s));
  int32_t rc = wait_event(ctx, ev, timeout_of(ctx));
  cudaEventDestroy(ev);
  if (rc) return rc;
  if (h.error) return OMG_E_OVERFLOW;
  return OMG_OK;
}

// ------------------------------------------------------------------ reverb
int32_t omg_estimate_reverb(omg_ctx* ctx, const float* bins, uint32_t n_bins, uint32_t nb, float bin_dt,
                            uint32_t n_jobs, omg_reverb* out) {
  if (!ctx || !bins || !out || !n_bins || n_bins > kMaxBins || !nb || nb > (uint32_t)MAXB || !n_jobs ||
      !(bin_dt > 0.0f))
    return OMG_E_INVALID;
  uint64_t per = (uint64_t)n_bins * nb, total = per * n_jobs;
  if (ctx->r_bins.n < total) CK(ctx->r_bins.alloc(total));
  if (ctx->r_jobs.n < n_jobs) {
    CK(ctx->r_jobs.alloc(n_jobs));
    CK(ctx->r_out.alloc(n_jobs));
  }
  std::vector<DReverbJob> rj(n_jobs);
  for (uint32_t i = 0; i < n_jobs; i++) {
    rj[i].bins_off = per * i;
    rj[i].n_bins = n_bins;
    rj[i].nb = nb;
    rj[i].bin_dt = bin_dt;
    rj[i].pad = 0;
  }
  cudaStream_t s = ctx->stream;
  CK(cudaMemcpyAsync(ctx->r_bins.p, bins, total * 4, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->r_jobs.p, rj.data(), n_jobs * sizeof(DReverbJob), cudaMemcpyHostToDevice, s));
  CK(launch_reverb(ctx->r_jobs.p, n_jobs, n_bins, ctx->r_bins.p, ctx->r_out.p, nullptr, s));
  CK(cudaMemcpyAsync(out, ctx->r_out.p, n_jobs * sizeof(omg_reverb), cudaMemcpyDeviceToHost, s));
  cudaEvent_t ev;
  CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  CK(cudaEventRecord(ev, s));
  int32_t rc = wait_event(ctx, ev, timeout_of(ctx));
  cudaEventDestroy(ev);
  return rc;
}

}  // extern "C"
