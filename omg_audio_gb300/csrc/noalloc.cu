// omg_trace_box_noalloc: the shoebox trace for callers that must not allocate.
//
// Some callers cannot call cudaMalloc: an audio render callback or any other
// real-time thread (an allocation can block for an unbounded time), code that
// runs while another component owns the device allocator, and hosts whose
// policy forbids allocations after start-up. For them this entry point runs
// the same trace kernel as omg_trace_box, but its scratch memory (the
// compensated histogram accumulators, the ray-queue head and error word, the
// segment counter, the job and wall-material records) lives in one
// file-scope device array of fixed size. The caller passes the job and its
// own device output buffers; the call allocates nothing and does not wait.
// The kernels' flag word (traversal stack, walk budget, loop guard) goes to
// the caller's optional device word flags_dev, written by the last kernel of
// the call: 0 when the trace ran to its end.
//
// Limits and sharing:
//  - n_bins * (n_bands + 3) <= OMG_NOALLOC_MAX_CELLS (larger jobs are rejected
//    with OMG_E_INVALID);
//  - the array is one per device, kept until the process exits, and shared by
//    every call: each call clears what must start at zero, and two calls that
//    overlap on the GPU (different streams, or different host threads without
//    ordering) race on it;
//  - the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress and loads every kernel the call may launch (the
//    trace kernel for 3 and 8 bands, with and without the near-tie rule), so
//    that no later call waits for the driver to load one (CUDA loads kernels
//    lazily by default); make that first call before any stream capture;
//  - the address is looked up once per device for the life of the process:
//    a cudaDeviceReset while this entry point is in use is not supported.
#include <cstring>
#include <mutex>

#include "omg_internal.h"
#include "scene.h"

namespace omg {

bool valid_material(const omg_material& m, uint32_t nb);   // api.cpp
bool finite3(const float* v);                               // api.cpp

namespace {

constexpr uint64_t kCells = OMG_NOALLOC_MAX_CELLS;
// layout (floats): accumulators 2 * kCells | DLaunch (4 words) | segments (4 words)
//                  | DJob | 6 DMat
constexpr uint64_t kAccFloats = 2 * kCells;
constexpr uint64_t kHdrOff = kAccFloats;
constexpr uint64_t kSegOff = kHdrOff + 4;
constexpr uint64_t kJobOff = kSegOff + 4;
constexpr uint64_t kJobFloats = (sizeof(DJob) + 15) / 16 * 4;
constexpr uint64_t kMatOff = kJobOff + kJobFloats;
constexpr uint64_t kTotalFloats = kMatOff + 6 * (sizeof(DMat) / 4);

static __device__ __align__(256) float g_noalloc_scratch[kTotalFloats];

struct WallMats {
  DMat m[6];
};

// the job and its wall materials arrive by value (kernel parameters) and are
// stored in the scratch array; the accumulators and counters are cleared
__global__ void noalloc_setup_kernel(float* scratch, DJob job, WallMats walls, uint32_t acc_floats) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  for (uint32_t i = tid; i < acc_floats; i += gridDim.x * blockDim.x) scratch[i] = 0.0f;
  if (tid == 0) {
    DLaunch* hdr = reinterpret_cast<DLaunch*>(scratch + kHdrOff);
    hdr->ray_counter = 0;
    hdr->error = 0;
    reinterpret_cast<uint32_t*>(scratch + kSegOff)[0] = 0;
    *reinterpret_cast<DJob*>(scratch + kJobOff) = job;
    DMat* m = reinterpret_cast<DMat*>(scratch + kMatOff);
    for (int w = 0; w < 6; w++) m[w] = walls.m[w];
  }
}

// (sum + comp) * 2^-64 into the caller's buffers (the accumulators are scaled,
// kAccScale), and the kernels' flag word into *flags (when given)
__global__ void noalloc_finalize_kernel(const float* scratch, uint32_t n_bins, uint32_t nb, float* bins,
                                        float* dirs, uint32_t* flags) {
  const uint32_t nbb = n_bins * nb, nd = n_bins * 3;
  if (flags && blockIdx.x == 0 && threadIdx.x == 0)
    *flags = reinterpret_cast<const DLaunch*>(scratch + kHdrOff)->error;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nbb + nd; i += gridDim.x * blockDim.x) {
    if (i < nbb) bins[i] = (scratch[i] + scratch[nbb + i]) * kAccUnscale;
    else dirs[i - nbb] = (scratch[2 * nbb + (i - nbb)] + scratch[2 * nbb + nd + (i - nbb)]) * kAccUnscale;
  }
}

constexpr int kMaxDevices = 64;
float* g_addr[kMaxDevices] = {};
int g_sms[kMaxDevices] = {};
std::mutex g_mu;

// Once per device, with that device current: the device address of the
// scratch array (the host-side symbol is only a stand-in, not an address).
cudaError_t scratch_for(int dev, float** out, int* n_sms) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    // load now every kernel a call may launch (lazy loading would otherwise
    // load each on its first launch, inside a caller's time-critical call)
    cudaFuncAttributes fa;
    if ((e = cudaFuncGetAttributes(&fa, noalloc_setup_kernel)) != cudaSuccess) return e;
    if ((e = cudaFuncGetAttributes(&fa, noalloc_finalize_kernel)) != cudaSuccess) return e;
    if ((e = preload_trace_kernels()) != cudaSuccess) return e;
    g_addr[dev] = static_cast<float*>(p);
    g_sms[dev] = sms;
  }
  *out = g_addr[dev];
  *n_sms = g_sms[dev];
  return cudaSuccess;
}

}  // namespace

}  // namespace omg

using namespace omg;

extern "C" int32_t omg_trace_box_noalloc(const omg_box_job* job, const omg_params* prm, float* bins_dev,
                                         float* dirs_dev, uint32_t* flags_dev, void* cuda_stream) {
  if (!job || !prm || !bins_dev || !dirs_dev) return OMG_E_INVALID;
  const uint32_t nb = prm->n_bands, n_bins = prm->n_bins;
  if (nb == 0 || nb > (uint32_t)MAXB || n_bins == 0 || job->n_rays == 0 || prm->dir_band >= nb ||
      !(prm->bin_dt > 0.0f) || !(prm->speed_of_sound > 0.0f))
    return OMG_E_INVALID;
  // the checks omg_trace_box makes on a box job: finite geometry and materials
  if (!finite3(job->src) || !finite3(job->lis) || !finite3(job->size)) return OMG_E_INVALID;
  for (int w = 0; w < 6; w++)
    if (!valid_material(job->walls[w], nb)) return OMG_E_INVALID;
  if ((uint64_t)n_bins * (nb + 3) > kCells) return OMG_E_INVALID;  // beyond the fixed scratch
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return OMG_E_DEVICE;
  }
  float* scratch = nullptr;
  int n_sms = 0;
  if (scratch_for(dev, &scratch, &n_sms) != cudaSuccess) {
    cudaGetLastError();
    return OMG_E_DEVICE;
  }
  // the job record, precomputed as omg_trace_box does (tracer.rs:90-95, 163)
  DJob d;
  std::memset(&d, 0, sizeof(d));
  d.geom = OMG_GEOM_BOX;
  d.n_rays = job->n_rays;
  d.seed = job->seed;
  for (int k = 0; k < 3; k++) {
    d.src[k] = job->src[k];
    d.lis[k] = job->lis[k];
    d.box[k] = job->size[k];
  }
  d.per_ray = 1.0f / (float)job->n_rays;
  d.floor_e = prm->energy_floor * d.per_ray;
  for (uint32_t b = 0; b < nb; b++) d.e0[b] = d.per_ray * job->energy[b];
  d.nb = nb;
  d.n_bins = n_bins;
  d.max_bounces = prm->max_bounces;
  d.dir_band = prm->dir_band;
  d.bin_dt = prm->bin_dt;
  d.max_time = prm->max_time;
  d.rr = prm->receiver_radius;
  d.wall_eps = prm->wall_eps;
  d.c = prm->speed_of_sound;
  d.box_mat = 0;
  d.ray_base = 0;
  d.acc_off = 0;
  d.out_off = 0;
  WallMats walls;
  for (int w = 0; w < 6; w++) walls.m[w] = make_dmat(job->walls[w], nb);

  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  const uint32_t acc = (uint32_t)(2ull * n_bins * (nb + 3));
  noalloc_setup_kernel<<<64, 256, 0, s>>>(scratch, d, walls, acc);
  LaunchShape shape;
  shape.loop_guard = prm->loop_guard;
  cudaError_t e = launch_trace(reinterpret_cast<const DJob*>(scratch + kJobOff), 1, job->n_rays, nb, nullptr,
                               reinterpret_cast<const DMat*>(scratch + kMatOff), nullptr, nullptr, scratch,
                               reinterpret_cast<DLaunch*>(scratch + kHdrOff),
                               reinterpret_cast<uint32_t*>(scratch + kSegOff), shape, n_sms, prm->tie_mode != 0, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return OMG_E_DEVICE;
  }
  noalloc_finalize_kernel<<<16, 256, 0, s>>>(scratch, n_bins, nb, bins_dev, dirs_dev, flags_dev);
  if (cudaGetLastError() != cudaSuccess) return OMG_E_DEVICE;
  return OMG_OK;
}
