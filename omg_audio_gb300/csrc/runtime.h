// Shared runtime types of the C ABI (api.cpp, api_scene.cpp, api_dome.cpp).
#pragma once
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "omg_internal.h"
#include "scene.h"

namespace omg {

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count) {
    release();
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e == cudaSuccess) n = count;
    else p = nullptr;
    return e;
  }
};

template <class T>
struct PinBuf {
  T* p = nullptr;
  size_t n = 0;
  ~PinBuf() { release(); }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count) {
    release();
    if (count == 0) count = 1;
    cudaError_t e = cudaMallocHost(&p, count * sizeof(T));
    if (e == cudaSuccess) n = count;
    else p = nullptr;
    return e;
  }
};

struct SceneRec {
  uint32_t n_tris = 0, n_prims = 0, n_nodes = 0, n_bands = 3;
  int32_t root = 0;
  uint32_t bvh_kind = OMG_BVH_SAH;
  DevBuf<float4> nodes, prims, normals;
  DevBuf<float4> nodes4;          // 4-wide collapse of `nodes` (host-built trees)
  DevBuf<float4> nodes4c;         // the same, child by child
  DevBuf<float4> nodes_f;         // binary nodes with grown boxes (fused multiply-add slab test)
  DevBuf<float4> prims_wt;        // watertight contexts: exact vertices A, B, C per primitive (prims' .w words)
  float fast_m[3] = {0, 0, 0};
  int32_t root4 = 0;
  uint32_t n_nodes4 = 0;
  DevBuf<DMat> mats;
  DevBuf<uint16_t> tri_surface;
  // host copies for export / queries
  std::vector<omg_material> materials;
  // per authored surface id, its first triangle's plane and material
  // (SurfaceTable::build, pt_mesh.rs:51-78): n[3], d, material, set
  struct SurfSeed {
    float n[3];
    float d;
    uint32_t mat;
    uint32_t set;
  };
  std::vector<SurfSeed> surf_seed;
  std::vector<float> ref_boxes;
  std::vector<uint32_t> ref_ab;
  std::vector<float> prim_geo;
  std::vector<uint32_t> prim_tri;
  std::vector<uint16_t> prim_mat;
};

struct BatchRec {
  uint32_t n_jobs = 0;
  uint32_t total_rays = 0;
  uint32_t max_nb = 0;
  uint32_t max_bins = 0;
  uint64_t n_out = 0, n_acc = 0, n_bin_floats = 0, n_dir_floats = 0;
  std::vector<DJob> jobs;
  std::vector<DMat> job_mats;
  std::vector<DPanel> panels;
  std::vector<DPanelGroup> groups;
  std::vector<DReverbJob> rjobs;
  DevBuf<DJob> d_jobs;
  DevBuf<DMat> d_job_mats;
  DevBuf<DPanel> d_panels;
  DevBuf<DPanelGroup> d_groups;
  DevBuf<float> d_acc, d_out;
  DevBuf<DLaunch> d_hdr;
  DevBuf<uint32_t> d_seg;
  DevBuf<DReverbJob> d_rjobs;
  DevBuf<omg_reverb> d_reverb;
  PinBuf<float> h_out;
  PinBuf<omg_reverb> h_reverb;
  PinBuf<DLaunch> h_hdr;
  PinBuf<uint32_t> h_seg;
  PinBuf<DJob> h_jobs;
  // wavefront rounds: per-ray state, two ray-id queues, control block
  DevBuf<float4> d_wf_pos, d_wf_dir, d_wf_e;
  DevBuf<uint32_t> d_wf_bounce, d_wf_queue;
  DevBuf<float2> d_wf_hit;
  DevBuf<WfCtl> d_wf_ctl;
  WfState wf{};
  bool coop_ok = false;           // near-tie rule and every mesh scene has a 4-wide tree (mode 2)
  DevBuf<uint32_t> d_ep_q;        // epoch queues (2 x rays)
  DevBuf<EpochCtl> d_ep_ctl;      // kMaxEpochs + 1 records
  LaunchShape shape;
  cudaGraphExec_t graph = nullptr;         // device-only launch
  cudaGraphExec_t graph_io = nullptr;      // H2D jobs + launch + D2H results
  cudaGraphExec_t graph_a = nullptr;       // clear + trace
  cudaGraphExec_t graph_b = nullptr;       // finalize + reverb
  cudaEvent_t done = nullptr;
  uint64_t signature = 0;
  ~BatchRec() {
    if (graph) cudaGraphExecDestroy(graph);
    if (graph_io) cudaGraphExecDestroy(graph_io);
    if (graph_a) cudaGraphExecDestroy(graph_a);
    if (graph_b) cudaGraphExecDestroy(graph_b);
    if (done) cudaEventDestroy(done);
  }
};

struct Ticket {
  std::unique_ptr<BatchRec> batch;
};

struct DomeRec;
struct MlpRec;
struct LateRec;
struct EarlyRec;

}  // namespace omg

struct omg_ctx {
  omg_params prm;
  int device = 0;
  int n_sms = 152;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  std::string last_error;
  uint32_t last_flags = 0;   // kernel flag word of the last trace or dome call (omg_last_flags)
  std::map<uint32_t, std::unique_ptr<omg::SceneRec>> scenes;
  uint32_t next_scene = 1;
  omg::DevBuf<omg::DScene> d_scenes;           // scene table indexed by scene id
  uint32_t scene_cap = 0;
  std::map<uint32_t, std::unique_ptr<omg::BatchRec>> batches;
  uint32_t next_batch = 1;
  std::unique_ptr<omg::BatchRec> cached;  // reused by the synchronous one-shot calls
  std::map<uint32_t, omg::Ticket> tickets;
  uint32_t next_ticket = 1;
  std::map<uint32_t, std::shared_ptr<omg::DomeRec>> probes;
  uint32_t next_probe = 1;
  std::map<uint32_t, std::shared_ptr<omg::MlpRec>> mlps;   // surrogate networks
  uint32_t next_mlp = 1;
  std::map<uint32_t, std::shared_ptr<omg::LateRec>> lates;  // late fields
  uint32_t next_late = 1;
  std::map<uint32_t, std::shared_ptr<omg::EarlyRec>> earlies;  // world early-reflection tables
  uint32_t next_early = 1;
  // raycast query scratch
  omg::DevBuf<float> q_o, q_d, q_t;
  omg::DevBuf<uint32_t> q_tri;
  omg::DevBuf<omg::DLaunch> q_hdr;
  omg::DevBuf<float> r_bins;
  omg::DevBuf<omg::DReverbJob> r_jobs;
  omg::DevBuf<omg_reverb> r_out;
  uint64_t last_h2d = 0, last_d2h = 0;     // copy volume of the last one-shot trace
  omg::LaunchShape shape;                  // launch shape for new batches (the autotuner's last pick)
};


namespace omg {

int32_t fail(omg_ctx* ctx, cudaError_t e, const char* where);
uint32_t timeout_of(const omg_ctx* ctx);
int32_t wait_event(omg_ctx* ctx, cudaEvent_t ev, uint32_t timeout_ms);
int32_t sync_scene_table(omg_ctx* ctx);
// The device view of an uploaded scene (one entry of the scene table).
DScene scene_view(const SceneRec& s, uint32_t walk_cap);
// api.cpp: a batch record for `jobs` (allocations, uploads, launch graphs);
// the same record refilled with new per-job values when the job layout
// (batch_layout) is unchanged; the kernels' error flags of its last read-back.
int32_t batch_prepare(omg_ctx* ctx, BatchRec& B, const omg_job* jobs, uint32_t n_jobs, const omg_panel* panels,
                      uint32_t n_panels);
int32_t batch_refill(omg_ctx* ctx, BatchRec& B, const omg_job* jobs, uint32_t n_jobs, const omg_panel* panels,
                     uint32_t n_panels);
uint64_t batch_layout(const omg_job* jobs, uint32_t n_jobs, uint32_t n_panels, const omg_params& P);
int32_t batch_flags(omg_ctx* ctx, const BatchRec& B);
constexpr uint32_t kMaxScenes = 4096;     // scene ids 1 .. kMaxScenes-1
bool valid_material(const omg_material& m, uint32_t nb);
bool finite3(const float* v);

}  // namespace omg

#define CK(call)                                            \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return omg::fail(ctx, e_, #call); \
  } while (0)
