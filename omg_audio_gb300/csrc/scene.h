// Host-side scene preparation (scene.cpp).
#pragma once
#include <cstdint>
#include <unordered_map>
#include <vector>

#include "omg_internal.h"

namespace omg {

constexpr float kMaxPrimEdge = 4.0f;  // mesh.rs:41

struct MeshBuilder {
  struct Key {
    int64_t x, y, z;
    bool operator==(const Key& o) const { return x == o.x && y == o.y && z == o.z; }
  };
  struct KeyHash {
    size_t operator()(const Key& k) const {
      uint64_t h = (uint64_t)k.x * 0x9E3779B97F4A7C15ULL;
      h ^= (uint64_t)k.y + 0x7F4A7C159E3779B9ULL + (h << 6) + (h >> 2);
      h ^= (uint64_t)k.z + 0x94D049BB133111EBULL + (h << 6) + (h >> 2);
      return (size_t)h;
    }
  };
  std::vector<float> positions;
  std::vector<uint32_t> indices;
  std::vector<uint16_t> tri_material;
  std::vector<omg_material> materials;
  std::vector<uint16_t> tri_surface;
  std::vector<float> tri_max_edge;
  float cur_max_edge = 0.0f;
  uint16_t next_surface = 0;
  std::unordered_map<Key, uint32_t, KeyHash> lookup;

  uint32_t material(const omg_material& m);
  uint32_t begin_surface();
  void coarse(float e) { cur_max_edge = e; }
  uint32_t vertex(const float p[3]);
  void tri(const float a[3], const float b[3], const float c[3], uint32_t m);
  void quad(const float a[3], const float b[3], const float c[3], const float d[3], uint32_t m);
  void abox(const float mn[3], const float mx[3], uint32_t m);
};

// prim_vtx (optional): the exact vertices a, b, c of every primitive (9 floats).
void tessellate(const float* pos, const uint32_t* idx, uint32_t n_tris, const uint16_t* tri_mat,
                const float* tri_max_edge, std::vector<float>& prim_geo, std::vector<uint32_t>& prim_tri,
                std::vector<uint16_t>& prim_mat, std::vector<float>* prim_vtx = nullptr);
// perm (optional): the tessellation index of the primitive at each leaf-order position.
void build_sah(std::vector<float>& prim_geo, std::vector<uint32_t>& prim_tri, std::vector<uint16_t>& prim_mat,
               std::vector<float>& ref_boxes, std::vector<uint32_t>& ref_ab, std::vector<uint32_t>* perm = nullptr);
// Binned SAH over all three axes (128 bins, leaves <= 4), same output form as
// build_sah; for walks under the near-tie rule, whose hit is tree-independent.
void build_sah3(std::vector<float>& prim_geo, std::vector<uint32_t>& prim_tri, std::vector<uint16_t>& prim_mat,
                std::vector<float>& ref_boxes, std::vector<uint32_t>& ref_ab, std::vector<uint32_t>* perm = nullptr);
// Returns the root ref; dev_nodes gets 16 floats per internal node.
int32_t flatten_bvh2(const std::vector<float>& ref_boxes, const std::vector<uint32_t>& ref_ab,
                     std::vector<float>& dev_nodes);
// The same tree with every node's children opened (largest surface area
// first) until it has 4: returns the root ref; dev_nodes gets 32 floats per
// node in the DScene::nodes4 layout; max_stack: the deepest traversal stack a
// walk of it can need.
int32_t flatten_bvh4(const std::vector<float>& ref_boxes, const std::vector<uint32_t>& ref_ab,
                     std::vector<float>& dev_nodes, uint32_t* max_stack);
// The binary nodes (flatten_bvh2 layout) with every child box grown by
// 2^-19 m[a] + pad on each side, rounded outward, where m[a] bounds
// |coordinate| along axis a of the scene (filled here: the largest |box
// coordinate| plus 1 m). The first term covers the rounding of the fused
// multiply-add slab test; pad (near_tie_pad) covers the hits Möller–Trumbore
// accepts just outside a triangle, so that walks on these boxes find every
// hit of every primitive.
void grow_nodes_for_fma(const std::vector<float>& dev_nodes, std::vector<float>& out, float m[3], float pad);
// The same growth on reference-form boxes (6 floats each).
void grow_ref_boxes(std::vector<float>& boxes, const float m[3], float pad);
// 2^-17 x the longest primitive edge (prim_geo: a, e1, e2 per primitive).
float near_tie_pad(const std::vector<float>& prim_geo);
void tri_normals(const float* pos, const uint32_t* idx, uint32_t n_tris, const uint16_t* tri_mat,
                 std::vector<float>& out);
DMat make_dmat(const omg_material& m, uint32_t nb);

}  // namespace omg
