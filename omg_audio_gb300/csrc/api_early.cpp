// C ABI of the GB300 tracer (include/omg_cuda.h), part 7: world early
// reflections (crates/omg-core/src/pt_mesh.rs; the WorldDiscovery and
// WorldSolve seams of crates/omg-scene/src/early_world.rs:18-48).
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "runtime.h"

using namespace omg;

namespace omg {

struct EarlyRec {
  uint32_t scene_id = 0;
  uint32_t n_surf = 0, base_overlay = 0, n_boxes = 0;
  float root_lo[3] = {0, 0, 0}, root_hi[3] = {0, 0, 0};
  DevBuf<DSurf> surf;
  DevBuf<float4> mtrans, boxes;
  DevBuf<uint32_t> err;
  // discovery scratch (grown on demand)
  uint32_t disc_rays = 0, tcap = 0;
  DevBuf<float> jitter;
  DevBuf<unsigned long long> cand_key, tkey;
  DevBuf<omg_chain> cand_chain, d_out;
  DevBuf<uint32_t> cand_slot, tidx, n_out;
  // solve scratch
  size_t src_cap = 0, chain_cap = 0, extra_cap = 0, rec_cap = 0;
  DevBuf<uint16_t> d_ids;
  DevBuf<float> d_pos;
  DevBuf<omg_chain> d_chains;
  DevBuf<omg_aabb> d_extras;
  DevBuf<omg_mesh_record> d_rec;
  PinBuf<uint32_t> h_word;         // [0] error bits, [1] discovered chains
  cudaEvent_t done = nullptr;
  ~EarlyRec() {
    if (done) cudaEventDestroy(done);
  }
};

}  // namespace omg

namespace {

// reflection_amplitude (material.rs:65-71) and the amplitude transmission
void amps(const omg_material& m, DSurf& s) {
  for (int b = 0; b < 3; b++) {
    s.refl[b] = std::sqrt(std::fmax(1.0f - m.absorption[b], 0.0f));
    s.trans[b] = m.transmission[b];
  }
}

EarlyRec* early_of(omg_ctx* ctx, uint32_t id) {
  auto it = ctx->earlies.find(id);
  return it == ctx->earlies.end() ? nullptr : it->second.get();
}

int32_t early_view(omg_ctx* ctx, const EarlyRec& R, DEarly& E) {
  auto it = ctx->scenes.find(R.scene_id);
  if (it == ctx->scenes.end()) return OMG_E_NOT_FOUND;
  std::memset(&E, 0, sizeof(E));
  E.S = scene_view(*it->second, ctx->prm.walk_budget);
  E.surf = R.surf.p;
  E.n_surf = R.n_surf;
  E.base_overlay = R.base_overlay;
  E.mtrans = R.mtrans.p;
  E.boxes = R.boxes.p;
  E.n_boxes = R.n_boxes;
  for (int a = 0; a < 3; a++) {
    E.root_lo[a] = R.root_lo[a];
    E.root_hi[a] = R.root_hi[a];
  }
  E.err = R.err.p;
  return OMG_OK;
}

// Read back the error word (and the chain count), wait for the stream with
// the context's bound, then clear the word; a set bit is a kernel-side
// overflow.
int32_t early_finish(omg_ctx* ctx, EarlyRec& R) {
  CK(cudaMemcpyAsync(R.h_word.p, R.err.p, 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(R.h_word.p + 1, R.n_out.p, 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaEventRecord(R.done, ctx->stream));
  int32_t rc = wait_event(ctx, R.done, timeout_of(ctx));
  if (rc) return rc;
  const uint32_t e = R.h_word.p[0];
  if (e) {
    CK(cudaMemset(R.err.p, 0, 4));
    ctx->last_error = "early reflections: kernel error bits " + std::to_string(e) +
                      " (1 stack, 2 crossing list, 4 walk budget, 8 chain table)";
    return OMG_E_OVERFLOW;
  }
  return OMG_OK;
}

uint32_t pow2_at_least(uint64_t v) {
  uint32_t p = 1;
  while (p < v && p < (1u << 31)) p <<= 1;
  return p;
}

}  // namespace

extern "C" {

int32_t omg_early_create(omg_ctx* ctx, uint32_t scene_id, const omg_panel* furniture, uint32_t n_furniture,
                         uint32_t* early_id) {
  if (!ctx || !early_id || (n_furniture && !furniture)) return OMG_E_INVALID;
  auto it = ctx->scenes.find(scene_id);
  if (it == ctx->scenes.end()) return OMG_E_NOT_FOUND;
  const SceneRec& S = *it->second;
  for (uint32_t i = 0; i < n_furniture; i++)
    if (!finite3(furniture[i].mn) || !finite3(furniture[i].mx)) return OMG_E_INVALID;
  const uint64_t n_surf = S.surf_seed.size() + 6ull * n_furniture;
  if (n_surf > 0xFFFFull) return OMG_E_INVALID;  // surface ids are u16, 0xFFFF meaning none
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, cudaGetLastError(), "cudaSetDevice");
  std::shared_ptr<EarlyRec> R(new EarlyRec());
  R->scene_id = scene_id;
  // SurfaceTable::build (pt_mesh.rs:51-78), then append_box (:86-109)
  std::vector<DSurf> tab;
  for (const SceneRec::SurfSeed& q : S.surf_seed) {
    DSurf s;
    std::memset(&s, 0, sizeof(s));
    s.n[0] = q.n[0];
    s.n[1] = q.n[1];
    s.n[2] = q.n[2];
    s.d = q.d;
    if (q.set) amps(S.materials[q.mat], s);
    tab.push_back(s);
  }
  R->base_overlay = (uint32_t)tab.size();
  std::vector<float4> bx;
  for (uint32_t i = 0; i < n_furniture; i++) {
    const omg_panel& f = furniture[i];
    for (int axis = 0; axis < 3; axis++) {
      for (int side = 0; side < 2; side++) {
        DSurf s;
        std::memset(&s, 0, sizeof(s));
        s.n[axis] = side == 0 ? -1.0f : 1.0f;
        const float* c = side == 0 ? f.mn : f.mx;
        s.d = s.n[0] * c[0] + s.n[1] * c[1] + s.n[2] * c[2];
        for (int k = 0; k < 3; k++) {
          s.fmin[k] = f.mn[k];
          s.fmax[k] = f.mx[k];
        }
        s.fmin[axis] = c[axis];
        s.fmax[axis] = c[axis];
        s.rect = 1u;
        amps(f.material, s);
        tab.push_back(s);
      }
    }
    bx.push_back(make_float4(f.mn[0], f.mn[1], f.mn[2], 0.0f));
    bx.push_back(make_float4(f.mx[0], f.mx[1], f.mx[2], 0.0f));
  }
  R->n_surf = (uint32_t)tab.size();
  R->n_boxes = n_furniture;
  std::vector<float4> mt;
  for (const omg_material& m : S.materials)
    mt.push_back(make_float4(m.transmission[0], m.transmission[1], m.transmission[2], 0.0f));
  // the root box of the tree: the bounds of every primitive (mesh.rs:300-313)
  const float FMAX = std::numeric_limits<float>::max();
  float lo[3] = {FMAX, FMAX, FMAX}, hi[3] = {-FMAX, -FMAX, -FMAX};
  for (size_t i = 0; i < S.prim_tri.size(); i++) {
    const float* g = &S.prim_geo[9 * i];
    for (int a = 0; a < 3; a++) {
      const float p0 = g[a], p1 = g[a] + g[3 + a], p2 = g[a] + g[6 + a];
      lo[a] = std::fmin(lo[a], std::fmin(std::fmin(p0, p1), p2));
      hi[a] = std::fmax(hi[a], std::fmax(std::fmax(p0, p1), p2));
    }
  }
  for (int a = 0; a < 3; a++) {
    R->root_lo[a] = lo[a];
    R->root_hi[a] = hi[a];
  }
  CK(R->surf.alloc(tab.size()));
  if (!tab.empty()) CK(cudaMemcpy(R->surf.p, tab.data(), tab.size() * sizeof(DSurf), cudaMemcpyHostToDevice));
  CK(R->mtrans.alloc(mt.size()));
  if (!mt.empty()) CK(cudaMemcpy(R->mtrans.p, mt.data(), mt.size() * sizeof(float4), cudaMemcpyHostToDevice));
  CK(R->boxes.alloc(bx.size()));
  if (!bx.empty()) CK(cudaMemcpy(R->boxes.p, bx.data(), bx.size() * sizeof(float4), cudaMemcpyHostToDevice));
  CK(R->err.alloc(1));
  CK(cudaMemset(R->err.p, 0, 4));
  CK(R->n_out.alloc(1));
  CK(cudaMemset(R->n_out.p, 0, 4));
  CK(R->h_word.alloc(2));
  CK(cudaEventCreateWithFlags(&R->done, cudaEventDisableTiming));
  const uint32_t id = ctx->next_early++;
  ctx->earlies[id] = R;
  *early_id = id;
  return OMG_OK;
}

int32_t omg_early_destroy(omg_ctx* ctx, uint32_t early_id) {
  if (!ctx) return OMG_E_INVALID;
  auto it = ctx->earlies.find(early_id);
  if (it == ctx->earlies.end()) return OMG_E_NOT_FOUND;
  cudaStreamSynchronize(ctx->stream);
  ctx->earlies.erase(it);
  return OMG_OK;
}

int32_t omg_early_info(omg_ctx* ctx, uint32_t early_id, uint32_t* base_overlay, uint32_t* n_surfaces) {
  if (!ctx) return OMG_E_INVALID;
  EarlyRec* R = early_of(ctx, early_id);
  if (!R) return OMG_E_NOT_FOUND;
  if (base_overlay) *base_overlay = R->base_overlay;
  if (n_surfaces) *n_surfaces = R->n_surf;
  return OMG_OK;
}

int32_t omg_early_discover(omg_ctx* ctx, uint32_t early_id, const float listener[3], uint32_t n_rays,
                           uint32_t rot, int32_t use_boxes, omg_chain* out, uint32_t cap, uint32_t* n_out) {
  if (!ctx || !listener || !n_out || (cap && !out) || !finite3(listener) || n_rays > (1u << 24))
    return OMG_E_INVALID;
  EarlyRec* R = early_of(ctx, early_id);
  if (!R) return OMG_E_NOT_FOUND;
  DEarly E;
  int32_t rc = early_view(ctx, *R, E);
  if (rc) return rc;
  const uint64_t n_cand = 3ull * n_rays;
  if (R->disc_rays < n_rays || R->disc_rays == 0) {
    const uint32_t nr = n_rays ? n_rays : 1u;
    CK(R->jitter.alloc(nr));
    CK(R->cand_key.alloc(3ull * nr));
    CK(R->cand_chain.alloc(3ull * nr));
    CK(R->cand_slot.alloc(3ull * nr));
    R->tcap = pow2_at_least(2ull * 3ull * nr);
    CK(R->tkey.alloc(R->tcap));
    CK(R->tidx.alloc(R->tcap));
    CK(R->d_out.alloc(3ull * nr));
    R->disc_rays = nr;
  }
  // the fan's jitter: one xorshift64* stream per rotation (pt_mesh.rs:393)
  std::vector<float> jit(n_rays);
  uint64_t st = (0xC6Bull ^ (uint64_t)rot) | 1ull;
  for (uint32_t i = 0; i < n_rays; i++) {
    uint64_t x = st;
    x ^= x >> 12;
    x ^= x << 25;
    x ^= x >> 27;
    st = x;
    jit[i] = (float)((x * 0x2545F4914F6CDD1DULL) >> 40) / (float)(1ull << 24);
  }
  if (n_rays)
    CK(cudaMemcpyAsync(R->jitter.p, jit.data(), n_rays * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemsetAsync(R->tkey.p, 0, (size_t)R->tcap * 8, ctx->stream));
  CK(cudaMemsetAsync(R->tidx.p, 0xFF, (size_t)R->tcap * 4, ctx->stream));
  CK(launch_early_discover(E, listener, n_rays, rot, use_boxes != 0, R->jitter.p, R->cand_key.p, R->cand_chain.p,
                           R->cand_slot.p, R->tkey.p, R->tidx.p, R->tcap, R->d_out.p, (uint32_t)n_cand, R->n_out.p,
                           ctx->stream));
  if ((rc = early_finish(ctx, *R))) return rc;
  const uint32_t n = R->h_word.p[1];
  const uint32_t w = n < cap ? n : cap;
  if (w) CK(cudaMemcpy(out, R->d_out.p, (size_t)w * sizeof(omg_chain), cudaMemcpyDeviceToHost));
  *n_out = n;
  return OMG_OK;
}

int32_t omg_early_solve(omg_ctx* ctx, uint32_t early_id, const uint16_t* source_ids, const float* source_pos,
                        uint32_t n_sources, const omg_chain* chains, uint32_t n_chains, const float listener[3],
                        const omg_aabb* extras, uint32_t n_extras, omg_mesh_record* out) {
  if (!ctx || !listener || !finite3(listener) || (n_sources && (!source_ids || !source_pos)) ||
      (n_chains && !chains) || (n_extras && !extras) || ((uint64_t)n_sources * n_chains != 0 && !out))
    return OMG_E_INVALID;
  for (uint32_t c = 0; c < n_chains; c++)
    if (chains[c].order > OMG_CHAIN_MAX_ORDER) return OMG_E_INVALID;
  for (uint32_t s = 0; s < n_sources; s++)
    if (!finite3(source_pos + 3 * s)) return OMG_E_INVALID;
  EarlyRec* R = early_of(ctx, early_id);
  if (!R) return OMG_E_NOT_FOUND;
  DEarly E;
  int32_t rc = early_view(ctx, *R, E);
  if (rc) return rc;
  const uint64_t n = (uint64_t)n_sources * n_chains;
  if (n == 0) return OMG_OK;
  if (R->src_cap < n_sources) {
    CK(R->d_ids.alloc(n_sources));
    CK(R->d_pos.alloc(3ull * n_sources));
    R->src_cap = n_sources;
  }
  if (R->chain_cap < n_chains) {
    CK(R->d_chains.alloc(n_chains));
    R->chain_cap = n_chains;
  }
  if (R->extra_cap < n_extras || R->extra_cap == 0) {
    CK(R->d_extras.alloc(n_extras ? n_extras : 1));
    R->extra_cap = n_extras ? n_extras : 1;
  }
  if (R->rec_cap < n) {
    CK(R->d_rec.alloc(n));
    R->rec_cap = n;
  }
  CK(cudaMemcpyAsync(R->d_ids.p, source_ids, n_sources * sizeof(uint16_t), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(R->d_pos.p, source_pos, 3ull * n_sources * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(R->d_chains.p, chains, n_chains * sizeof(omg_chain), cudaMemcpyHostToDevice, ctx->stream));
  if (n_extras)
    CK(cudaMemcpyAsync(R->d_extras.p, extras, n_extras * sizeof(omg_aabb), cudaMemcpyHostToDevice, ctx->stream));
  CK(launch_early_solve(E, R->d_ids.p, R->d_pos.p, n_sources, R->d_chains.p, n_chains, listener, R->d_extras.p,
                        n_extras, R->d_rec.p, ctx->stream));
  if ((rc = early_finish(ctx, *R))) return rc;
  CK(cudaMemcpy(out, R->d_rec.p, n * sizeof(omg_mesh_record), cudaMemcpyDeviceToHost));
  return OMG_OK;
}

}  // extern "C"
