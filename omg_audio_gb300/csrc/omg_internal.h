// Device-side layout shared by the host runtime (api.cpp, scene.cpp) and the
// kernels (trace.cu, dome.cu, lbvh.cu, reverb.cu).
//
// HBM layout of one scene (all 16-byte aligned, read through the read-only
// path):
//   nodes   : BVH2 with both child boxes in the parent, 64 B per node
//             n0 = (c0.lo.x, c0.lo.y, c0.lo.z, c0.hi.x)
//             n1 = (c0.hi.y, c0.hi.z, c1.lo.x, c1.lo.y)
//             n2 = (c1.lo.z, c1.hi.x, c1.hi.y, c1.hi.z)
//             n3 = (c0 ref, c1 ref, -, -) as int bits
//             ref >= 0: internal node index; ref < 0: leaf ~((start << 3) | (count - 1))
//   prims   : 48 B per tessellated primitive, in leaf order
//             p0 = (a.xyz, material id)  p1 = (e1.xyz, original tri id)  p2 = (e2.xyz, surface id)
//   normals : 16 B per ORIGINAL triangle: normalize(e1 x e2) of the authored triangle
//             (mesh.rs:458-461), .w = material id
//   mats    : 80 B per material, with the branch weights precomputed (bit-identical
//             to computing them per bounce: same f32 operations, same order)
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/omg_cuda.h"

namespace omg {

constexpr int MAXB = OMG_MAX_BANDS;
constexpr int STACK_DEPTH = 64;
// Histogram bins of one echogram at most: the reverb estimate holds one band's
// curve (an FP64 and an f32 value a bin) in a block's 227 KB of shared memory.
constexpr uint32_t kMaxBins = 19370;           // mesh.rs:492 (64-entry traversal stack)

// tracer.rs:148-182 per material: p = clamp(max_b T_b^2, 0.02, 0.5) when
// > 1e-5 else 0; transmitted weight T_b^2 / p; reflected weight
// max(1 - a_b - T_b^2, 0) / (1 - p).
struct alignas(16) DMat {
  float p;
  float scattering;
  float wt[MAXB];
  float wr[MAXB];
  float absorption[MAXB];      // dome escape: tp *= 1 - absorption (dome.rs:365-367)
  float t2[MAXB];              // dome through: tp *= T^2 (dome.rs:398-402)
  float pad[2];
};
static_assert(sizeof(DMat) == 144, "DMat layout");

struct DScene {
  const float4* nodes;
  const float4* prims;
  const float4* normals;
  const DMat* mats;
  const uint16_t* tri_surface;   // authored surface id per original tri (segment_hits merge)
  int32_t root;                  // root ref (internal 0, or a leaf ref)
  uint32_t n_nodes;
  uint32_t n_prims;
  uint32_t n_bands;
  // The same tree collapsed to 4 children per node (host-built scenes only;
  // null otherwise). 128 B per node, 8 float4:
  //   lo.x[4] hi.x[4] lo.y[4] hi.y[4] lo.z[4] hi.z[4] ref[4] (int bits) -
  // refs as in `nodes`; an unused child slot has ref kEmpty4 and a zero box.
  const float4* nodes4;
  int32_t root4;
  uint32_t n_nodes4;
  // The 4-wide tree once more, child by child for walks that split a node's
  // children over 4 lanes: 32 B per child, child k of node n at float4 index
  // 8 n + 2 k: (lo.x, lo.y, lo.z, hi.x), (hi.y, hi.z, ref bits, 0).
  const float4* nodes4c;
  // `nodes` with every child box grown by 2^-19 M_a + pad on each side (M_a:
  // the scene's largest |coordinate| along axis a, plus 1 m; pad: 2^-17 x the
  // longest primitive edge), for the near-tie walks: the fused multiply-add
  // slab test of walks whose origin lies within |o_a| <= 7 M_a
  // (device_common.cuh:ray_aabb_fma), and a margin that holds every hit
  // Möller–Trumbore accepts just outside a triangle; null: a leaf root.
  const float4* nodes_f;
  float fast_m[3];
  // Node and leaf visits one closest-hit walk may take before it stops and
  // flags error 4: every node is entered at most once per pass, so a longer walk
  // means a corrupt tree. walk_budget = min(2 n_nodes + n_prims + 64, the
  // context's omg_params.walk_budget); walk_budget4 the same for the 4-wide tree
  // (n_nodes4 + 1).
  uint32_t walk_budget;
  uint32_t walk_budget4;
  // Watertight contexts (omg_params.tri_test): the exact vertices A, B, C of
  // every primitive as (A, material), (B, triangle), (C, surface), the same
  // .w words as prims; the closest-hit walks then test these with the
  // watertight test. Null: the reference's test on prims.
  const float4* prims_wt;
};
constexpr int32_t kEmpty4 = 0x7FFFFFFE;

// Panel overlay (scene.rs:90-137): box, an index into the batch's material
// table, and the panel's index in the caller's order (exact-tie rule).
struct alignas(16) DPanel {
  float mn[3];
  uint32_t mat;
  float mx[3];
  uint32_t orig;
};

// Up to 4 spatially close panels of one job behind their union box.
struct alignas(16) DPanelGroup {
  float mn[3];
  uint32_t first;   // into the batch's panel array
  float mx[3];
  uint32_t count;
};

// One job of a launch. Values that the reference computes per ray from
// constants are precomputed here with the same f32 operations.
struct alignas(16) DJob {
  uint32_t geom;          // OMG_GEOM_BOX / OMG_GEOM_MESH
  uint32_t scene;         // index into the scene table
  uint32_t n_rays;
  uint32_t seed;
  float src[3];
  float per_ray;          // 1 / n_rays (tracer.rs:90)
  float lis[3];
  float floor_e;          // energy_floor * per_ray (tracer.rs:163)
  float box[3];
  uint32_t box_mat;       // first of 6 wall materials in the batch material table
  float e0[MAXB];         // per_ray * source_energy[b] (tracer.rs:95)
  uint32_t nb;
  uint32_t n_bins;
  uint32_t max_bounces;
  uint32_t dir_band;
  float bin_dt;
  float max_time;
  float rr;               // receiver radius
  float wall_eps;
  float c;                // speed of sound
  uint32_t panel_off;
  uint32_t n_panels;
  uint32_t group_off;     // panel groups of this job
  uint32_t n_groups;
  uint32_t ray_base;      // first global ray id of this job
  uint64_t acc_off;       // float offset of this job's accumulators
  uint64_t out_off;       // float offset of this job's output (bins then dirs)
};

// Per-launch header in device memory (scratch: cleared before every launch).
struct alignas(16) DLaunch {
  uint32_t ray_counter;   // persistent-queue head
  uint32_t error;         // kernel flags: 1 stack overflow, 2 crossing list overflow, 4 walk budget,
                          // 8 persistent-kernel loop guard
  uint32_t pad[2];
};

// Histogram accumulators hold values scaled by 2^64 (exact): the float
// atomics flush subnormals, and scaled values of energies down to 2^-149 stay
// normal. Finalizing multiplies by 2^-64, exact wherever the result is normal.
constexpr float kAccScale = 18446744073709551616.0f;        // 2^64
constexpr float kAccUnscale = 5.42101086242752217e-20f;     // 2^-64
// Accumulator block of one job (all float, compensated pairs):
//   bins_s[n_bins*nb], bins_c[n_bins*nb], dirs_s[n_bins*3], dirs_c[n_bins*3]
inline uint64_t acc_floats(uint32_t n_bins, uint32_t nb) { return 2ull * n_bins * (nb + 3); }
inline uint64_t out_floats(uint32_t n_bins, uint32_t nb) { return 1ull * n_bins * (nb + 3); }

// Launch shapes of the tracer kernel (autotuned).
struct LaunchShape {
  uint32_t block_threads = 256;
  uint32_t blocks_per_sm = 4;
  uint32_t refill_min = 1;      // a warp refetches rays once this many lanes are idle
  uint32_t walk_steps = 0;      // traversal steps per lane per loop iteration (0 = a whole walk)
  uint32_t shade_min = 32;      // lanes that shade together (or every waiting lane once none walks)
  uint32_t mode = 0;            // persistent kernel: 0 lane state machine, 1 warp-local wavefront,
                                // 2 cooperative 4-lane walks
  uint32_t tail_mode = 0;       // the persistent kernel of epochs after the first
  uint32_t wide = 0;            // persistent walks on the 4-wide tree (near-tie rule only)
  // mode 2: the persistent kernel walks each ray with 4 lanes (one child of a
  // 4-wide node each) and shades wl_shade_min rays at a time (near-tie rule, every
  // mesh scene of the batch host-built)
  uint32_t wf_iters = 0;        // wavefront rounds before the persistent kernel takes over (0: none)
  uint32_t wf_tail = 0;         // ... or as soon as at most this many rays are alive
  uint32_t epochs = 0;          // persistent-kernel epochs (0: one launch that never parks)
  uint32_t park_pct = 50;       // an epoch parks its rays once at most this % of them remain
  uint32_t park_min = 4096;     // epochs of at most this many rays run to the end
  uint32_t wl_shade_min = 32;   // modes 1 and 2: rays a warp shades together once that many wait
  uint32_t loop_guard = 0;      // loop iterations of one warp of a persistent kernel before it stops
                                // and flags error 8 (0: kDefaultLoopGuard); from omg_params.loop_guard
};
constexpr uint32_t kDefaultLoopGuard = 1u << 22;

// Wavefront state (wavefront.cu). One record per ray of the batch, indexed by
// the ray's global id, holds everything the bounce loop carries from one
// segment to the next; two queues hold the ids of the live rays.
struct alignas(16) WfCtl {
  uint32_t count[2];     // queue lengths
  uint32_t tail;         // 1 once the persistent kernel takes over
  uint32_t tail_q;       // the queue it resumes from
  uint32_t tail_n;       // and its length
  uint32_t pad[3];
};
struct WfState {
  float4* pos;           // p.xyz, distance travelled
  float4* dir;           // d.xyz, ray stream state (uint bits)
  float4* e;             // band energies 0-3 at [r], 4-7 at [cap + r]
  uint32_t* bounce;      // segments traced so far
  float2* hit;           // closest mesh hit: t, primitive index bits (-1: none)
  uint32_t* queue;       // queue 0 at [0, cap), queue 1 at [cap, 2 cap)
  WfCtl* ctl;
  uint32_t cap;          // rays of the batch
};

// Epochs of the persistent kernel. As rays end, the lanes of the persistent
// kernel go idle; an epoch therefore stops once few of its rays remain: every
// lane parks its ray at the end of its current segment (state saved in the
// WfState records, id appended to the next epoch's queue) and the next epoch
// resumes the parked rays in full warps. One record per epoch, cleared
// before the launch.
struct alignas(16) EpochCtl {
  uint32_t n;            // rays queued for this epoch (appended by the previous one)
  uint32_t fetch;        // queue head
  uint32_t ended;        // rays of this epoch that ended
  uint32_t park;         // 1: park rays at their next segment end
};
constexpr uint32_t kMaxEpochs = 32;
struct EpochArgs {
  const uint32_t* in_q;  // ray ids of this epoch (cur->n of them); null: fresh rays 0 .. total_rays-1
  uint32_t* out_q;       // the next epoch's queue; null: every ray runs to its end
  EpochCtl* cur;         // null: a single launch (fresh rays, header ray counter, no parking)
  EpochCtl* next;
  uint32_t park_pct;
  uint32_t park_min;
  WfState st;            // per-ray records (saved and restored state)
  uint32_t max_loop;     // the persistent kernels' per-warp loop guard (error 8)
};

// ----------------------------------------------------------- kernel launchers
// trace.cu. `ep`: one epoch of an epoch chain (null: a single launch).
// wt: the context's scenes carry exact vertices (watertight test)
cudaError_t launch_trace(const DJob* jobs, uint32_t n_jobs, uint32_t total_rays, uint32_t max_nb,
                         const DScene* scenes, const DMat* job_mats, const DPanel* panels,
                         const DPanelGroup* groups, float* acc,
                         DLaunch* hdr, uint32_t* job_segments, const LaunchShape& shape, int n_sms, bool tie,
                         cudaStream_t s, const EpochArgs* ep = nullptr, bool wt = false);
// trace.cu: load the per-lane trace kernel variants launch_trace may pick for a
// single launch (3 and 8 bands, with and without the near-tie rule) now, so
// that a later launch does not wait for the driver's lazy module loading.
cudaError_t preload_trace_kernels();
// coop.cu: the mode-2 persistent kernel (same arguments as launch_trace).
cudaError_t launch_trace_coop(const DJob* jobs, uint32_t n_jobs, uint32_t total_rays, uint32_t max_nb,
                              const DScene* scenes, const DMat* job_mats, const DPanel* panels,
                              const DPanelGroup* groups, float* acc, DLaunch* hdr, uint32_t* job_segments,
                              const LaunchShape& shape, int n_sms, const EpochArgs& ea, cudaStream_t s);
// wavefront.cu: wavefront rounds (when shape.wf_iters > 0), then the
// persistent kernel on the remaining rays, in shape.epochs epochs (ep_q: two
// queues of st.cap ids; ep_ctl: kMaxEpochs + 1 records, cleared).
cudaError_t launch_wavefront(const DJob* jobs, uint32_t n_jobs, uint32_t total_rays, uint32_t max_nb,
                             const DScene* scenes, const DMat* job_mats, const DPanel* panels,
                             const DPanelGroup* groups, float* acc, DLaunch* hdr, uint32_t* job_segments,
                             const WfState& st, uint32_t* ep_q, EpochCtl* ep_ctl, const LaunchShape& shape,
                             int n_sms, bool tie, cudaStream_t s, bool wt = false);
cudaError_t launch_finalize(const DJob* jobs, uint32_t n_jobs, const float* acc, float* out, uint64_t total_out,
                            cudaStream_t s);
cudaError_t launch_raycast(const DScene* scene, const float* o, const float* d, uint32_t n, float* t,
                           uint32_t* tri, DLaunch* hdr, bool tie, cudaStream_t s);
// reverb.cu: one echogram per job at out + out_off (bins part), n_bins x nb
struct DReverbJob {
  uint64_t bins_off;
  uint32_t n_bins;
  uint32_t nb;
  float bin_dt;
  uint32_t pad;
};
cudaError_t launch_reverb(const DReverbJob* rj, uint32_t n_jobs, uint32_t max_bins, const float* bins,
                          omg_reverb* out, const uint32_t* job_segments, cudaStream_t s);
// late.cu: blend each traced slot's fresh echogram (a batch output at
// fresh + fresh_off) into the slot's average, then its reverb (rj: the slots'
// echograms in avg, one per update) and state.
struct DLateUpdate {
  uint32_t slot;
  uint32_t tick;
  uint64_t fresh_off;
  float alpha;          // EMA weight of the fresh echogram
  uint32_t pad;
};
cudaError_t launch_late_update(const DLateUpdate* up, uint32_t n_up, const float* fresh, float* avg,
                               uint32_t* version, const DReverbJob* rj, omg_reverb* rev, omg_late_state* state,
                               uint32_t n_bins, uint32_t nb, uint32_t from_bin, uint32_t dir_band, cudaStream_t s);
// lbvh.cu: build the node array for prims already in device memory; reorders
// prims into leaf order (prims_out) and returns the root ref.
cudaError_t lbvh_build(const float4* prims_in, uint32_t n_prims, float4* prims_out, float4* nodes_out,
                       int32_t* root_ref, void* scratch, size_t scratch_bytes, cudaStream_t s);
size_t lbvh_scratch_bytes(uint32_t n_prims);
// sah3.cu: the three-axis binned-SAH tree of build_sah3 (scene.cpp), built on
// the GPU from the primitives in tessellation order (prims: a, e1, e2 per
// primitive, 3 float4 each). Returns the tree in build_sah3's form and
// numbering (ref_boxes: 6 floats a node, ref_ab: children or leaf range) and
// perm[i] = the tessellation index of the primitive at leaf-order position i.
cudaError_t sah3_build_device(const float4* prims, uint32_t n_prims, std::vector<float>& ref_boxes,
                              std::vector<uint32_t>& ref_ab, std::vector<uint32_t>& perm, cudaStream_t s);
// DScene::nodes_f from `nodes` on the device (m: the bound of |coordinate| per
// axis; pad: near_tie_pad of the primitives)
cudaError_t grow_nodes(const float4* nodes, float4* out, uint32_t n_nodes, const float m[3], float pad,
                       cudaStream_t s);

// dome.cu
struct DDomePanel {
  int32_t axis;
  float plane, lat0, lat1, z0, z1;
  int32_t glass;
  float t2[MAXB];         // trans^2 per band
};
struct DDomeLaunch {
  const DScene* scene;
  const float4* fan;      // n_fan directions (xyz, bin index in w)
  uint32_t n_fan;
  uint32_t n_rays;
  uint32_t max_events;
  uint32_t nb;
  const DDomePanel* panels;   // glass first, then leaves
  uint32_t n_glass;
  uint32_t n_panels;
  const float* eyes;          // n_eyes x 3
  uint32_t n_eyes;
  float* ray_tp;              // n_eyes x n_rays x nb
  uint8_t* ray_escape;        // n_eyes x n_rays
  float* ema;                 // n_eyes x 9 x nb (device state)
  uint32_t* primed;           // n_eyes
  float* raw;                 // n_eyes x 9 x nb
  float* out_dir;             // n_eyes x 9 x 3
  float* out_energy;          // n_eyes x 9 x nb
  DLaunch* hdr;
  uint32_t* events;           // escape events + through calls (2 counters)
  uint32_t tie;               // near-tie rule of the escape raycasts (omg_params.tie_mode)
  uint32_t wt;                // the scene carries exact vertices (watertight test)
};
cudaError_t launch_dome(const DDomeLaunch& L, cudaStream_t s);

// mlp.cu: tensor-core GEMM D[M x N] = A[M x K] . B[N x K]^T (bf16 in, f32
// accumulate) with strided operands and a fused epilogue.
struct GemmArgs {
  const void* A;            // __nv_bfloat16; element (m, k) at A[m a_rs + k a_ks]
  int64_t a_rs, a_ks;
  const void* B;            // element (n, k) at B[n b_rs + k b_ks]
  int64_t b_rs, b_ks;
  uint32_t M, N, K;
  uint32_t n_tile;          // columns per CTA: multiple of 16, <= 256
  const float* bias;        // [N] or null
  float* D;                 // f32 [M x ldd] or null
  int64_t ldd;
  uint32_t accumulate;      // 1: D += (atomically; K split over grid z)
  float* Z;                 // pre-activation f32 or null
  int64_t ldz;
  void* Y;                  // __nv_bfloat16 activation out or null
  int64_t ldy;
  void* Yt;                 // the same activation transposed (element (m, n) at Yt[n ldyt + m]) or null
  int64_t ldyt;
  uint32_t act;             // 0 none, 1 GELU (tanh form)
  uint32_t* err;            // error word: 16 = an mbarrier wait ran out
};
size_t gemm_smem_bytes();
cudaError_t gemm_init();
cudaError_t launch_gemm(const GemmArgs& g, uint32_t k_split, cudaStream_t s);
// backward elementwise on 32 x 32 tiles: mode 0 the MSE loss gradient of
// P = outputs against Q = targets (weights w per column, nullable; loss +=),
// mode 1 dZ = P (dA) * GELU'(Q (Z)); writes dZ, its bf16 copy and transpose,
// and adds the column sums into gb (zeroed by the caller)
cudaError_t launch_grad_tile(uint32_t mode, const float* P, const float* Q, const float* w, uint32_t rows,
                             uint32_t cols, float* dZ, void* dZh, void* dZht, float* gb, float* loss, cudaStream_t s);
// AdamW of every layer of one ensemble member in one launch
struct AdamwLayer {
  float *W, *mW, *vW, *b, *mb, *vb;
  const float *gW, *gb;
  void *Wh, *Wht;
  uint32_t in, out;
  uint64_t off;             // first element of this layer in the launch's index space (W then b)
};
constexpr int kMaxAdamwLayers = 17;
struct AdamwTable {
  AdamwLayer L[kMaxAdamwLayers];
  uint32_t n;
  uint64_t total;
};
cudaError_t launch_adamw_all(const AdamwTable& tab, const float* sched, const uint32_t* step, float b1, float b2,
                             float eps, float wd, cudaStream_t s);
// inputs (bf16 copy + transpose) and targets (f32) of this step's batch rows
cudaError_t launch_gather_pair(const float* X, uint32_t xcols, const float* Y, uint32_t ycols, const uint32_t* perm,
                               const uint32_t* step, uint32_t spe, uint32_t rows, void* xh, void* xht, float* t,
                               cudaStream_t s);
cudaError_t launch_step(uint32_t* step, cudaStream_t s);
cudaError_t launch_to_bf16_t(const float* x, uint32_t rows, uint32_t cols, void* xh, void* xht, cudaStream_t s);
cudaError_t launch_standardize(const float* x, const float* mean, const float* sd, uint32_t cols, uint64_t n,
                               void* out, cudaStream_t s);
cudaError_t launch_ensemble(const float* y, const float* mean, const float* sd, uint32_t cols, uint64_t n,
                            float* acc, float* acc2, bool first, bool last, float inv_e, cudaStream_t s);
cudaError_t launch_row_spread(const float* mean, const float* sd, uint32_t cols, uint32_t rows, float level,
                              float* out, cudaStream_t s);
cudaError_t build_dome_fan(float4* fan, uint32_t n_fan, cudaStream_t s);

// early.cu: world early reflections (pt_mesh.rs). One surface of the table
// (pt_mesh.rs:30-41): plane n.x = d, per-band reflection and transmission
// amplitudes, and for a furniture face its rect.
struct alignas(16) DSurf {
  float n[3];
  float d;
  float refl[3];
  uint32_t rect;
  float trans[3];
  float pad0;
  float fmin[3];
  float pad1;
  float fmax[3];
  float pad2;
};
struct DEarly {
  DScene S;                   // the mesh (its binary tree: first-found closest hits, segment walks)
  const DSurf* surf;
  uint32_t n_surf;
  uint32_t base_overlay;
  const float4* mtrans;       // per scene material: amplitude transmission of bands 0..2
  const float4* boxes;        // furniture boxes: 2 float4 (min, max) each
  uint32_t n_boxes;
  float root_lo[3], root_hi[3];  // the tree's root box (segment_hits tests it first)
  uint32_t* err;              // error bits: 1 stack, 2 crossing list, 4 walk budget, 8 hash table
};
// Discovery: n_rays fan rays -> 3 candidates each (cand_key 0 = none), the
// first occurrence of every key (hash table tkey/tidx of tcap slots, cleared
// to 0 / 0xFFFFFFFF) compacted in candidate order into out (<= cap), *n_out.
cudaError_t launch_early_discover(const DEarly& E, const float lis[3], uint32_t n_rays, uint32_t rot, bool use_boxes,
                                  const float* jitter, unsigned long long* cand_key, omg_chain* cand_chain,
                                  uint32_t* cand_slot, unsigned long long* tkey, uint32_t* tidx, uint32_t tcap,
                                  omg_chain* out, uint32_t cap, uint32_t* n_out, cudaStream_t s);
cudaError_t launch_early_solve(const DEarly& E, const uint16_t* ids, const float* pos, uint32_t n_src,
                               const omg_chain* chains, uint32_t n_chains, const float lis[3], const omg_aabb* extras,
                               uint32_t n_extras, omg_mesh_record* out, cudaStream_t s);

}  // namespace omg
