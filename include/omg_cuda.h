/*
 * omg_cuda.h — C ABI of the GB300 stochastic energy path tracer.
 *
 * Drop-in for omg-audio's late-field backend seam (crates/omg-scene/src/late.rs)
 * and its ambient dome (crates/omg-scene/src/dome.rs). Plain C types only: a
 * Rust `extern "C"` block, ctypes, or any FFI binds it directly.
 *
 * Conventions (every entry point):
 *  - returns int32_t status: OMG_OK (0), OMG_PENDING (>0), or a negative error;
 *  - never panics, never blocks without a bound (waits take a timeout);
 *  - never retains caller pointers past the call;
 *  - a context is used by one thread at a time (the reference serialises its
 *    backends behind one global Mutex, late.rs:51,93; do the same).
 * All buffers passed in are HOST memory unless the name says `_dev`.
 */
#ifndef OMG_CUDA_H
#define OMG_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OMG_ABI_VERSION 3
#define OMG_MAX_BANDS 8
#define OMG_DOME_BINS 9          /* dome.rs:30: 8 azimuth sectors + zenith */

/* status codes */
#define OMG_OK 0
#define OMG_PENDING 1            /* async result not ready (poll again) */
#define OMG_E_INVALID (-1)       /* bad argument */
#define OMG_E_OOM (-2)           /* device or host allocation failed */
#define OMG_E_DEVICE (-3)        /* CUDA error; the context is unusable */
#define OMG_E_TIMEOUT (-4)       /* a bounded wait ran out */
#define OMG_E_OVERFLOW (-5)      /* traversal stack / crossing list overflow (kernel flag) */
#define OMG_E_NOT_FOUND (-6)     /* unknown scene / probe / ticket id */
#define OMG_E_NO_DEVICE (-7)     /* no usable CUDA device */

/* BVH builders for omg_scene_upload */
#define OMG_BVH_SAH 0            /* the reference's binned-SAH tree (mesh.rs:241-405), built on the host */
#define OMG_BVH_LBVH 1           /* Morton/Karras LBVH built on the GPU */
#define OMG_BVH_SAH3 2           /* binned SAH over all three axes (128 bins, leaves <= 4), built on the GPU:
                                    fewer node visits than OMG_BVH_SAH; hits equal the reference tree's under
                                    the near-tie rule (tie_mode 1), exact ties may resolve differently without it */
#define OMG_BVH_SAH3_HOST 3      /* the same tree built on the host (same nodes, boxes and leaf ranges; the
                                    primitives inside a leaf may be in another order) */

typedef struct omg_ctx omg_ctx;

/* Per-band surface acoustics: crates/omg-core/src/material.rs:7-16 (NBANDS
 * there is 3; here the band count is a runtime value <= 8). Amplitude
 * transmission T: the energy fraction is T*T. */
typedef struct omg_material {
    float absorption[OMG_MAX_BANDS];
    float scattering;
    float transmission[OMG_MAX_BANDS];
} omg_material;

/* Tracer constants made runtime values. Defaults (omg_params_default) are the
 * reference constants: tracer.rs:12-16 (BIN_DT 0.010, MAX_TIME 3.0,
 * NBINS 300, RECEIVER_RADIUS 0.5, WALL_EPS 1e-3), 64 bounces (tracer.rs:103),
 * energy floor 1e-7 x per-ray energy (tracer.rs:163,179), c = 343 (lib.rs:18),
 * 3 bands (lib.rs:22), direction band 1 (tracer.rs:123-125). */
typedef struct omg_params {
    uint32_t n_bands;
    uint32_t n_bins;             /* at most 19,370 (the reverb estimate holds one band's curve in
                                    shared memory): omg_create, a job or omg_estimate_reverb asking
                                    for more is refused (NULL / OMG_E_INVALID) */
    float bin_dt;
    float max_time;
    uint32_t max_bounces;
    float energy_floor;
    float receiver_radius;
    float wall_eps;
    float speed_of_sound;
    uint32_t dir_band;
    int32_t device;              /* CUDA device ordinal */
    uint32_t timeout_ms;         /* bound on every wait (0 = 10000) */
    uint32_t tie_mode;           /* closest hit among near-ties (relative t-gap < 1e-6):
                                    0 = the first one found in the reference's traversal
                                    order (mesh.rs:505, strict <); 1 = the lowest authored
                                    surface id, then triangle id (precision-independent) */
    /* Device-side limits. Each ends the kernel's work early with a flag, so no
     * kernel can spin; a call whose kernels raised a flag returns OMG_E_OVERFLOW
     * and omg_last_flags() gives the flags. The context stays usable. */
    uint32_t walk_budget;        /* node and leaf visits of one closest-hit walk before it stops
                                    (flag 4); 0 = 2 x nodes + primitives + 64, which no walk of
                                    a sound tree reaches. Smaller values cap it. */
    uint32_t loop_guard;         /* loop iterations of one warp of a persistent trace kernel
                                    before it stops (flag 8); 0 = 2^22 */
    uint32_t tri_test;           /* ray-triangle test of the closest-hit queries: OMG_TRI_REFERENCE
                                    or OMG_TRI_WATERTIGHT (needs tie_mode 1; omg_create returns
                                    NULL otherwise) */
} omg_params;

/* Ray-triangle tests (omg_params.tri_test) */
#define OMG_TRI_REFERENCE 0      /* the reference's Moller-Trumbore with its epsilons (mesh.rs:437-456)
                                    on a, b - a, c - a: hits equal the reference's */
#define OMG_TRI_WATERTIGHT 1     /* Woop, Benthin, Wald 2013 on the exact vertices: a ray through an edge
                                    or vertex shared by two triangles hits one of them; scenes uploaded
                                    to such a context keep the vertices beside the primitives (48 B a
                                    primitive). The dome's straight-through seep and the early
                                    reflections keep the reference's test. */

/* LateBackend::trace job (late.rs:28-40): analytic shoebox [0,size]^3, walls in
 * Shoebox order x-,x+,y-,y+,z-,z+ (scene.rs:23-26). */
typedef struct omg_box_job {
    float size[3];
    omg_material walls[6];
    float src[3];
    float lis[3];
    uint32_t n_rays;
    float energy[OMG_MAX_BANDS];
    uint32_t seed;               /* per-ray stream seed (see omg_trace_box) */
} omg_box_job;

/* Panel overlay box (scene.rs:90-137; late.rs:88 `panels: &[(Vec3, Vec3, Material)]`). */
typedef struct omg_panel {
    float mn[3];
    float mx[3];
    omg_material material;
} omg_panel;

/* WorldLateBackend::trace_world job (late.rs:81-91) over an uploaded mesh. */
typedef struct omg_world_job {
    float src[3];
    float lis[3];
    uint32_t n_rays;
    float energy[OMG_MAX_BANDS];
    uint32_t seed;
} omg_world_job;

/* One job of a batch: either geometry kind, its own rays, bands and histogram
 * length (the per-job values override omg_params). */
#define OMG_GEOM_BOX 0
#define OMG_GEOM_MESH 1
typedef struct omg_job {
    uint32_t geom;               /* OMG_GEOM_BOX or OMG_GEOM_MESH */
    uint32_t scene_id;           /* OMG_GEOM_MESH: an uploaded scene */
    float box_size[3];           /* OMG_GEOM_BOX */
    omg_material box_walls[6];   /* OMG_GEOM_BOX */
    float src[3];
    float lis[3];
    uint32_t n_rays;
    float energy[OMG_MAX_BANDS];
    uint32_t seed;
    uint32_t n_bands;            /* 0 = context default */
    uint32_t n_bins;             /* 0 = context default */
    float max_time;              /* 0 = context default */
    uint32_t panel_offset;       /* into the batch's panel array */
    uint32_t n_panels;
} omg_job;

/* estimate_reverb output (tracer.rs:204-257, params.rs:17-37) plus the
 * least-squares T20 fit of the FP64 Schroeder curve and the segment count. */
typedef struct omg_reverb {
    float rt60[OMG_MAX_BANDS];
    float level[OMG_MAX_BANDS];
    float rt60_fit[OMG_MAX_BANDS];
    uint64_t segments;           /* ray segments traced for this job */
} omg_reverb;

/* Ambient-dome panel (dome.rs:41-69) with its per-band AMPLITUDE transmission:
 * a pane (glass=1) passes rays with T^2 (glass_transmission, walkthrough.rs:310-320);
 * a door leaf (glass=0) blocks escapes and seeps T^2 straight through
 * (DOOR/HEAVY_PANEL_TRANSMISSION, walkthrough.rs:322-326). */
typedef struct omg_dome_panel {
    int32_t axis;                /* 0: plane of constant x, 1: constant y */
    float plane;
    float lat0, lat1;
    float z0, z1;
    int32_t glass;
    float trans[OMG_MAX_BANDS];
} omg_dome_panel;

typedef struct omg_dome_bin {    /* dome.rs:71-77 */
    float dir[3];
    float energy[OMG_MAX_BANDS];
} omg_dome_bin;

/* ------------------------------------------------------------------ context */

/* Fill the reference defaults. */
void omg_params_default(omg_params* p);

/* Create a context on p->device. NULL = no usable device: the caller keeps the
 * CPU path (GpuTracer::new -> Option, crates/omg-gpu/src/lib.rs:33-37). */
omg_ctx* omg_create(const omg_params* p);
void omg_destroy(omg_ctx* ctx);
int32_t omg_abi_version(void);
const char* omg_status_string(int32_t status);
/* Last CUDA error text of the context (empty when none). */
const char* omg_last_error(const omg_ctx* ctx);
/* Kernel flag word of the context's last trace or dome call that read one
 * back: 0 = none; 1 traversal stack overflow, 2 crossing list overflow,
 * 4 walk budget (omg_params.walk_budget), 8 persistent-kernel loop guard
 * (omg_params.loop_guard). Any flag makes that call return OMG_E_OVERFLOW. */
uint32_t omg_last_flags(const omg_ctx* ctx);
/* Change the context's device-side limits (omg_params.walk_budget and
 * loop_guard; 0 = default) for every later call, batches already created
 * included. Waits for the context's stream first. */
int32_t omg_set_limits(omg_ctx* ctx, uint32_t walk_budget, uint32_t loop_guard);
/* Launch work of this context on a caller stream (a cudaStream_t; NULL = the
 * context's own stream). */
int32_t omg_set_stream(omg_ctx* ctx, void* cuda_stream);

/* ------------------------------------------------------------- mesh builder */
/* Incremental mesh assembly with 0.1 mm vertex dedup: MeshBuilder,
 * crates/omg-core/src/mesh.rs:70-165. */
typedef struct omg_mesh_builder omg_mesh_builder;
omg_mesh_builder* omg_mb_create(void);
void omg_mb_destroy(omg_mesh_builder* mb);
uint32_t omg_mb_material(omg_mesh_builder* mb, const omg_material* m);     /* mesh.rs:93-96 */
uint32_t omg_mb_begin_surface(omg_mesh_builder* mb);                       /* mesh.rs:103-106 */
void omg_mb_coarse(omg_mesh_builder* mb, float max_edge);                  /* mesh.rs:132-134 */
void omg_mb_tri(omg_mesh_builder* mb, const float a[3], const float b[3], const float c[3], uint32_t material); /* :116-126 */
void omg_mb_quad(omg_mesh_builder* mb, const float a[3], const float b[3], const float c[3], const float d[3],
                 uint32_t material);                                       /* mesh.rs:137-140 */
void omg_mb_abox(omg_mesh_builder* mb, const float mn[3], const float mx[3], uint32_t material); /* :144-153 */
/* Bulk form: quad i has corners q[12i..12i+11]; begin_surface is called
 * new_surface[i] times first; coarse(max_edge[i]) applies before it (NULL arrays skip). */
void omg_mb_quads(omg_mesh_builder* mb, const float* q, const uint16_t* material, const uint8_t* new_surface,
                  const float* max_edge, uint32_t n);
void omg_mb_counts(const omg_mesh_builder* mb, uint32_t* n_verts, uint32_t* n_tris, uint32_t* n_materials);
void omg_mb_export(const omg_mesh_builder* mb, float* positions, uint32_t* indices, uint16_t* tri_material,
                   uint16_t* tri_surface, float* tri_max_edge);

/* ------------------------------------------------------------------- scenes */
/* Upload a mesh and build its BVH (MeshBuilder::build + GpuMeshTracer::new,
 * mesh.rs:155-221, omg-gpu/src/lib.rs:274-287). Oversized triangles are
 * tessellated exactly as mesh.rs:241-287; hits report the ORIGINAL triangle id.
 * n_bands fixes the band count of this scene's materials. */
int32_t omg_scene_upload(omg_ctx* ctx, const float* positions, uint32_t n_verts, const uint32_t* indices,
                         uint32_t n_tris, const uint16_t* tri_material, const float* tri_max_edge,
                         const omg_material* materials, uint32_t n_materials, uint32_t n_bands,
                         uint32_t bvh_kind, uint32_t* scene_id);
/* Same, straight from a builder. */
int32_t omg_scene_from_builder(omg_ctx* ctx, const omg_mesh_builder* mb, uint32_t n_bands, uint32_t bvh_kind,
                               uint32_t* scene_id);
int32_t omg_scene_release(omg_ctx* ctx, uint32_t scene_id);
/* Node / primitive counts of an uploaded scene. */
int32_t omg_scene_info(omg_ctx* ctx, uint32_t scene_id, uint32_t* n_nodes, uint32_t* n_prims, uint32_t* n_tris);
/* The uploaded BVH in the reference's flattened form (mesh.rs:463-481,
 * omg-gpu/src/layout.rs:96-122): nodes {bmin[3], a, bmax[3], b} as boxes[n*6]
 * + ab[n*2], prims {a, e1, e2} as geo[p*9] + tri[p] + material[p]. */
int32_t omg_scene_export_bvh(omg_ctx* ctx, uint32_t scene_id, float* node_boxes, uint32_t* node_ab,
                             float* prim_geo, uint32_t* prim_tri, uint16_t* prim_mat);

/* ---------------------------------------------------------------- tracing */
/* The stream: ray r of a job draws from PCG-RXS-M-XS seeded
 * (seed ^ r*0x9E3779B9) + 1 with two warm-up draws
 * (crates/omg-gpu/shaders/trace_mesh.wgsl:90-105, 211-213).
 * Outputs: bins[n_bins*n_bands] (bin-major), dirs[n_bins*3], FP32 values of
 * compensated (two-float) sums. The caller's buffers are overwritten, as the
 * reference clears the Echogram first (tracer.rs:89). */

/* LateBackend::trace (late.rs:28-40, omg-gpu/src/lib.rs:1051-1068). */
int32_t omg_trace_box(omg_ctx* ctx, const omg_box_job* job, float* bins, float* dirs, omg_reverb* reverb);

/* WorldLateBackend::trace_world (late.rs:81-91, omg-gpu/src/lib.rs:845-874)
 * over WithPanels{mesh, panels} (scene.rs:90-137). */
int32_t omg_trace_world(omg_ctx* ctx, uint32_t scene_id, const omg_world_job* job, const omg_panel* panels,
                        uint32_t n_panels, float* bins, float* dirs, omg_reverb* reverb);

/* Many jobs (uneven rays, bands, histogram lengths, scenes) in one persistent
 * launch captured in a CUDA graph. bins/dirs are the jobs' outputs back to
 * back, in job order; reverb (nullable) gets one entry per job. */
int32_t omg_trace_batch(omg_ctx* ctx, const omg_job* jobs, uint32_t n_jobs, const omg_panel* panels,
                        uint32_t n_panels, float* bins, float* dirs, omg_reverb* reverb);

/* Device-resident batches: upload once, launch many times, read back. */
int32_t omg_batch_create(omg_ctx* ctx, const omg_job* jobs, uint32_t n_jobs, const omg_panel* panels,
                         uint32_t n_panels, uint32_t* batch_id);
/* Launch on the context stream without host copies or waits (stream order). */
int32_t omg_batch_launch(omg_ctx* ctx, uint32_t batch_id);
/* The same launch in two parts (part 1: clear scratch + trace kernel; part 2:
 * finalize + reverb kernels; part 0: both), for timing the trace kernel alone. */
int32_t omg_batch_launch_part(omg_ctx* ctx, uint32_t batch_id, uint32_t part);
/* Host->device and device->host bytes copied by the last one-shot trace call
 * (omg_trace_box / omg_trace_world / omg_trace_batch). */
int32_t omg_io_bytes(omg_ctx* ctx, uint64_t* h2d, uint64_t* d2h);
/* Wait (bounded) and copy results to host; any pointer may be NULL. */
int32_t omg_batch_read(omg_ctx* ctx, uint32_t batch_id, float* bins, float* dirs, omg_reverb* reverb);
/* Float counts of one batch's bins and dirs outputs. */
int32_t omg_batch_sizes(omg_ctx* ctx, uint32_t batch_id, uint64_t* n_bin_floats, uint64_t* n_dir_floats);
/* Total segments traced by the last launch of the batch (device counter). */
int32_t omg_batch_segments(omg_ctx* ctx, uint32_t batch_id, uint64_t* segments);
int32_t omg_batch_destroy(omg_ctx* ctx, uint32_t batch_id);
/* Number of kernel launches one omg_batch_launch issues. */
int32_t omg_batch_kernel_count(omg_ctx* ctx, uint32_t batch_id, uint32_t* n_kernels);

/* Asynchronous form of the seam (LateBackend::poll_into, late.rs:42-48):
 * submit returns a ticket at once; poll returns OMG_PENDING until done. */
int32_t omg_submit_world(omg_ctx* ctx, uint32_t scene_id, const omg_world_job* job, const omg_panel* panels,
                         uint32_t n_panels, uint32_t* ticket);
int32_t omg_poll(omg_ctx* ctx, uint32_t ticket, float* bins, float* dirs, omg_reverb* reverb);

/* Launch shape of a batch's trace. Rays first run `wf_rounds` wavefront
 * rounds (a traversal kernel and a shading kernel over a queue of live rays);
 * once at most `wf_tail` rays are alive, or after the last round, the
 * persistent kernel finishes them, in `epochs` launches: an epoch parks its
 * rays between two segments once at most `park_pct` % of them remain, and the
 * next epoch resumes them in full warps (the last one runs every ray to its
 * end). wf_rounds = 0 and epochs = 0: one persistent launch. The result is
 * the same for every shape.
 * Autotuner: times the persistent kernel's shapes (threads per block x blocks
 * per SM x refill threshold x walk steps x shading group), then epoch counts and park
 * thresholds, then wavefront round counts and hand-over thresholds; keeps the
 * fastest for the batch and as the context's default for later batches. */
typedef struct omg_tune_result {
    uint32_t block_threads;
    uint32_t blocks_per_sm;
    uint32_t refill_min;         /* a warp refills from the ray queue once this many lanes idle */
    uint32_t walk_steps;         /* traversal steps per lane per loop iteration (0 = whole walk) */
    uint32_t shade_min;          /* lanes of a warp that shade together (1..32; 0 reads as 1) */
    uint32_t mode;               /* persistent kernel: 0 per-lane state machine, 1 warp-local wavefront
                                    (walks refill lane by lane; rays shade wl_shade_min at a time), 2 the same with
                                    each walk split over 4 lanes of a 4-wide tree (tie_mode 1 and
                                    host-built trees; otherwise mode 0 runs) */
    uint32_t tail_mode;          /* persistent kernel of epochs after the first (same values) */
    uint32_t wide;               /* 1: persistent walks use the 4-wide tree (tie_mode 1, host-built trees) */
    uint32_t wf_rounds;          /* wavefront rounds before the persistent kernel (0 = none) */
    uint32_t wf_tail;            /* hand over to the persistent kernel at <= this many live rays */
    uint32_t epochs;             /* persistent-kernel epochs, <= 32 (0 = one launch) */
    uint32_t park_pct;           /* an epoch parks its rays once <= this % of them remain */
    uint32_t wl_shade_min;       /* modes 1 and 2: rays a warp shades together once that many wait
                                    (1..32, 0 reads as 32; every waiting ray once none walks) */
    float ms;                    /* autotune: mean time of the clear + trace part */
} omg_tune_result;
int32_t omg_batch_autotune(omg_ctx* ctx, uint32_t batch_id, uint32_t reps, omg_tune_result* best);
/* Set a batch's shape by hand (block_threads a multiple of 32, <= 256;
 * block_threads x blocks_per_sm <= 2048; refill_min in 1..32); it also
 * becomes the context's default. get: the batch's current shape (ms = 0). */
int32_t omg_batch_set_shape(omg_ctx* ctx, uint32_t batch_id, const omg_tune_result* shape);
int32_t omg_batch_get_shape(omg_ctx* ctx, uint32_t batch_id, omg_tune_result* shape);

/* ----------------------------------------------------------- mesh queries */
/* Closest hit per ray (Mesh::raycast, mesh.rs:484-541): t (-1 on miss) and the
 * ORIGINAL triangle id (0xFFFFFFFF on miss). */
int32_t omg_raycast(omg_ctx* ctx, uint32_t scene_id, const float* origins, const float* dirs, uint32_t n,
                    float* t, uint32_t* tri);

/* ------------------------------------------------------------------- reverb */
/* estimate_reverb (tracer.rs:204-257) of n_jobs echograms back to back on the
 * GPU: FP64 Schroeder integral, 2-point -5/-25 dB slope, least-squares fit. */
int32_t omg_estimate_reverb(omg_ctx* ctx, const float* bins, uint32_t n_bins, uint32_t n_bands, float bin_dt,
                            uint32_t n_jobs, omg_reverb* out);

/* --------------------------------------------------------------------- dome */
/* DomeProbe::new over an uploaded world mesh (dome.rs:312-326): n_fan
 * golden-spiral directions (384 in the reference), fixed glass panes. */
int32_t omg_dome_create(omg_ctx* ctx, uint32_t scene_id, const omg_dome_panel* glass, uint32_t n_glass,
                        uint32_t n_fan, uint32_t n_bands, uint32_t* probe_id);
int32_t omg_dome_destroy(omg_ctx* ctx, uint32_t probe_id);
/* DomeProbe::sample (dome.rs:424-478) for n_eyes listener positions at once.
 * out: n_eyes x 9 bins (EMA'd, 0.35; the first call primes with 1.0);
 * raw_energy (nullable): n_eyes x 9 x n_bands energies before the EMA;
 * escape (nullable): n_eyes x n_rays per-ray sky-escape flags (1 = escaped);
 * ray_tp (nullable): n_eyes x n_rays x n_bands per-ray throughput.
 * Every listener keeps its own EMA state inside the probe (slot = eye index). */
int32_t omg_dome_sample(omg_ctx* ctx, uint32_t probe_id, const float* eyes, uint32_t n_eyes,
                        const omg_dome_panel* leaves, uint32_t n_leaves, uint32_t n_rays, uint32_t max_events,
                        omg_dome_bin* out, float* raw_energy, uint8_t* escape, float* ray_tp);
/* The same sample in two calls, so that it can overlap other work (a batch
 * trace on another stream): submit enqueues the inputs, the kernels and the
 * result copies on cuda_stream (NULL: the context's stream) and returns at
 * once; collect waits (bounded by omg_params.timeout_ms) and copies the
 * results out. `want` selects the optional outputs collect may return:
 * 1 raw_energy, 2 escape, 4 ray_tp. One sample per probe may be in flight. */
#define OMG_DOME_WANT_RAW 1u
#define OMG_DOME_WANT_ESCAPE 2u
#define OMG_DOME_WANT_TP 4u
int32_t omg_dome_submit(omg_ctx* ctx, uint32_t probe_id, const float* eyes, uint32_t n_eyes,
                        const omg_dome_panel* leaves, uint32_t n_leaves, uint32_t n_rays, uint32_t max_events,
                        uint32_t want, void* cuda_stream);
int32_t omg_dome_collect(omg_ctx* ctx, uint32_t probe_id, omg_dome_bin* out, float* raw_energy, uint8_t* escape,
                         float* ray_tp);
/* Work of the probe's last sample: trace_escape events (dome.rs:333-380) and
 * trace_through calls (dome.rs:390-422), summed over listeners. */
int32_t omg_dome_segments(omg_ctx* ctx, uint32_t probe_id, uint64_t* escape_events, uint64_t* through_calls);

/* -------------------------------------------------------------- late field */
/* The consumer side of the seam (Sim::reverb_world / reverb_only,
 * sim.rs:330-398) for many sim instances at once. Each slot keeps its
 * averaged echogram (Sim::echo_avg) in device memory. A tick traces the
 * slots the caller's gates fired for in ONE batched launch; then, on the
 * device, each traced slot's echogram is blended in (Echogram::ema,
 * tracer.rs:46-57, with the caller's weight) and its
 * reverb (estimate_reverb) and late direction (late_direction,
 * tracer.rs:59-77, from dir_from_s on, energy of the context's dir_band) are
 * computed. Only the slot states travel back. The trace gate, the per-tick
 * budget and the staleness compensation (sim.rs:38-75, 364-395) stay with the
 * caller, which knows the poses.
 * Slots share the context's n_bins and n_bands; a submitted job must use
 * them. One tick is in flight per field: submit returns OMG_PENDING while the
 * previous tick has not been polled to completion. */
typedef struct omg_late_state {
    float rt60[OMG_MAX_BANDS];   /* estimate_reverb of the averaged echogram */
    float level[OMG_MAX_BANDS];
    float dir[3];                /* unit direction of the late arrivals (1,0,0 when none) */
    float anisotropy;            /* 0 diffuse .. 1 all from one direction */
    uint32_t version;            /* updates blended in so far (0: never traced) */
    uint32_t updated_tick;       /* the tick of the last update */
} omg_late_state;
int32_t omg_late_create(omg_ctx* ctx, uint32_t n_slots, float dir_from_s, uint32_t* field_id);
int32_t omg_late_destroy(omg_ctx* ctx, uint32_t field_id);
/* Enqueue one tick on the context stream: trace jobs[i] for slot slots[i]
 * (distinct slots), then blend each into its slot with weight alpha[i]
 * (NULL: 1 on the slot's first update, 0.3 after). Returns at once; *tick
 * numbers the tick (1, 2, ...). n_jobs = 0 enqueues only the state read-back. */
int32_t omg_late_submit(omg_ctx* ctx, uint32_t field_id, const uint32_t* slots, const omg_job* jobs,
                        const float* alpha, uint32_t n_jobs, const omg_panel* panels, uint32_t n_panels,
                        uint32_t* tick);
/* OMG_PENDING until the last submitted tick is done; then every slot's state
 * (n_slots records) and that tick's number. Without a tick in flight: the
 * last states. */
int32_t omg_late_poll(omg_ctx* ctx, uint32_t field_id, omg_late_state* states, uint32_t* tick);
/* Forget a slot's history (a new sim instance in it): its next update
 * replaces the echogram (alpha 1). Not while a tick is in flight. */
int32_t omg_late_reset(omg_ctx* ctx, uint32_t field_id, uint32_t slot);
/* A slot's averaged echogram (n_bins x n_bands, n_bins x 3). Not while a tick is in flight. */
int32_t omg_late_read(omg_ctx* ctx, uint32_t field_id, uint32_t slot, float* bins, float* dirs);

/* ---------------------------------------------- world early reflections */
/* Specular surface chains over the world mesh (crates/omg-core/src/pt_mesh.rs):
 * discovery from the listener (mesh_chains, :382-457; the WorldDiscovery seam,
 * omg-scene/src/early_world.rs:18-26, kernel K3 in the reference's GPU plan)
 * and the exact per-(source, chain) solve with transmission along every leg
 * (mesh_record, :186-337; the WorldSolve seam, early_world.rs:36-48, kernel
 * K4). A chain lists authored surface ids listener-first; surfaces at or above
 * the table's base_overlay are the faces of the furniture boxes, 6 per box in
 * the order x-min, x-max, y-min, y-max, z-min, z-max (SurfaceTable::append_box,
 * pt_mesh.rs:86-109). Closest hits follow the reference's first-found order
 * (tie_mode 0 semantics) whatever the context's tie_mode; over the reference's
 * tree (OMG_BVH_SAH) they are the reference's hits exactly. */
#define OMG_CHAIN_MAX_ORDER 3
#define OMG_NO_SURF 0xFFFFu
typedef struct omg_chain {       /* MChain (pt_mesh.rs:111) */
    uint16_t surf[OMG_CHAIN_MAX_ORDER];  /* OMG_NO_SURF beyond order */
    uint16_t order;              /* 0 = the direct path */
} omg_chain;
typedef struct omg_aabb {        /* pt.rs:31-35: a transient blocker (door leaf, pane, furniture) */
    float mn[3];
    float mx[3];
    float transmission[3];       /* per-band amplitude through it */
} omg_aabb;
typedef struct omg_mesh_record { /* MeshRecord (pt_mesh.rs:113-121) */
    uint16_t source;
    uint16_t chain[OMG_CHAIN_MAX_ORDER];
    uint32_t order;
    float delay_s;
    float dir[3];                /* from the listener toward the image source */
    float gains[3];              /* per-band amplitude */
    uint32_t key;                /* MeshRecord::key (pt_mesh.rs:123-134) */
    uint32_t valid;              /* 0: the pair does not solve (mesh_record -> None) */
} omg_mesh_record;
/* SurfaceTable::build over an uploaded scene plus append_box per furniture box
 * (early_world.rs:114-120); the boxes also reflect discovery rays. Scenes of at
 * most 2^16 - 1 surfaces (ids are u16). */
int32_t omg_early_create(omg_ctx* ctx, uint32_t scene_id, const omg_panel* furniture, uint32_t n_furniture,
                         uint32_t* early_id);
int32_t omg_early_destroy(omg_ctx* ctx, uint32_t early_id);
int32_t omg_early_info(omg_ctx* ctx, uint32_t early_id, uint32_t* base_overlay, uint32_t* n_surfaces);
/* WorldDiscovery::discover / mesh_chains: n_rays fan rays from the listener,
 * fan rotation rot, up to 3 specular bounces each; the unique chains in the
 * reference's first-found order (ray, then bounce). use_boxes = 0 leaves the
 * furniture out (the furniture switch off). *n_out = the number found; the
 * first min(n_out, cap) are written. */
int32_t omg_early_discover(omg_ctx* ctx, uint32_t early_id, const float listener[3], uint32_t n_rays,
                           uint32_t rot, int32_t use_boxes, omg_chain* out, uint32_t cap, uint32_t* n_out);
/* WorldSolve::solve_batch / mesh_record for every (source, chain) pair in one
 * launch: out[s * n_chains + c]. extras: blockers every leg pays when it
 * passes through them (mesh_record's `extras`). */
int32_t omg_early_solve(omg_ctx* ctx, uint32_t early_id, const uint16_t* source_ids, const float* source_pos,
                        uint32_t n_sources, const omg_chain* chains, uint32_t n_chains, const float listener[3],
                        const omg_aabb* extras, uint32_t n_extras, omg_mesh_record* out);

/* ------------------------------------------------------------- wire formats */
/* The web bridge's flat trace jobs, as the wasm build queues them for its GPU
 * driver and the driver reads them (crates/omg-web/src/lib.rs:150-202 and
 * 365-416; web/gpu.js:181-199 packJob, 420-437 pumpWorldLate), traced here as
 * ONE batch instead of one dispatch per job. Word values are converted as the
 * driver's Uint32Array stores do (JavaScript ToUint32: truncate, modulo 2^32).
 * Box job, 57 f32: [0] sim id, [1] n_rays, [2] seed, [3..6] room size,
 *   [6..9] source, [9..12] listener, [12..15] band energy, [15..57] 6 walls
 *   (x-,x+,y-,y+,z-,z+) x (absorption x3, scattering, transmission x3).
 * World job, 1034 f32 (10 + 64 x 16): [0] sim id, [1] n_rays, [2] seed,
 *   [3..6] source, [6..9] listener, [9] n_panels (<= 64), [10..] panels of
 *   16 f32: min xyz, scattering, max xyz, 0, absorption xyz, 0,
 *   transmission xyz, 0; unit band energy (gpu.js:434).
 * echo: per job the injection record of lib.rs:158/204-218: n_bins x 3 bin
 *   energies, then n_bins x 3 direction sums (1800 f32 at the reference's
 *   300 bins). ids (nullable): the jobs' sim ids. reverb (nullable): one per job.
 * The context must run 3 bands (the formats' NBANDS); n_floats must be a
 * whole number of jobs. */
#define OMG_WEB_BOX_JOB_F32S 57
#define OMG_WEB_BOX_JOB_VERSION 2        /* lib.rs:158 GPU_JOB_VERSION */
#define OMG_WEB_WORLD_MAX_PANELS 64
#define OMG_WEB_WORLD_JOB_F32S (10 + OMG_WEB_WORLD_MAX_PANELS * 16)
#define OMG_WEB_WORLD_JOB_VERSION 3      /* lib.rs:377 WLATE_VERSION */
int32_t omg_trace_web_box_jobs(omg_ctx* ctx, const float* jobs, uint32_t n_floats, float* echo, uint32_t* ids,
                               omg_reverb* reverb);
int32_t omg_trace_web_world_jobs(omg_ctx* ctx, uint32_t scene_id, const float* jobs, uint32_t n_floats,
                                 float* echo, uint32_t* ids, omg_reverb* reverb);

/* The simulation -> renderer contract in its flat f32 form (ParamBlock,
 * crates/omg-core/src/params.rs:57-141): [0] version, [1] n_taps,
 * [2..8] reverb rt60[3], level[3], [8] remote flag, [9..24] remote rt60[3],
 * send[3], sh[9], then 9 f32 per tap: key, delay_s, dir[3], gains[3], 0.
 * Host-only (no device work). */
#define OMG_PARAM_FLAT_HEADER 24
#define OMG_PARAM_FLAT_PER_TAP 9
typedef struct omg_tap {         /* params.rs:7-16 */
    uint32_t key;
    float delay_s;
    float dir[3];
    float gains[3];
} omg_tap;
typedef struct omg_param_block { /* params.rs:57-66, taps passed beside it */
    uint64_t version;
    float rt60[3];               /* ReverbParams (params.rs:18-29) */
    float level[3];
    int32_t has_remote;          /* RemoteReverb (params.rs:44-55) present */
    float remote_rt60[3];
    float remote_send[3];
    float remote_sh[9];
} omg_param_block;
/* ParamBlock::flat_len (params.rs:75-77). */
uint32_t omg_param_block_flat_len(uint32_t n_taps);
/* ParamBlock::write_flat (params.rs:79-106): out_len >= flat_len(n_taps). */
int32_t omg_param_block_write_flat(const omg_param_block* pb, const omg_tap* taps, uint32_t n_taps, float* out,
                                   uint32_t out_len);
/* ParamBlock::read_flat (params.rs:108-141). *n_taps gets the block's tap
 * count; taps beyond max_taps, or a block longer than len, give OMG_E_INVALID
 * (the reference panics on a short slice). */
int32_t omg_param_block_read_flat(const float* data, uint32_t len, omg_param_block* pb, omg_tap* taps,
                                  uint32_t max_taps, uint32_t* n_taps);
/* The reverb part of n ParamBlocks from late-field slot states (bands 0..2 of
 * rt60 and level, as Sim writes estimate_reverb into its block,
 * sim.rs:364-398); version = the slot's update count; no remote field. */
int32_t omg_param_block_from_late(const omg_late_state* states, uint32_t n, omg_param_block* out);

/* --------------------------------------------------------------- surrogate */
/* No counterpart in the reference: the learned surrogate of the tracer. An
 * ensemble of `members` MLPs n_in -> hidden (x n_hidden, GELU) -> n_out,
 * trained on the GPU with tensor-core (tcgen05) BF16 GEMMs accumulating in
 * FP32, FP32 master weights and AdamW. Inputs and targets are standardized
 * per column from the training data. */
typedef struct omg_mlp_config {
    uint32_t n_in;               /* 38 for the room surrogate */
    uint32_t hidden;             /* multiple of 16, <= 256 */
    uint32_t n_hidden;           /* hidden layers (4) */
    uint32_t n_out;              /* <= 256 (192 = 64 log-time bins x 3 bands) */
    uint32_t members;            /* ensemble size, 1..16: their spread is the uncertainty */
    uint32_t seed;               /* weight init */
} omg_mlp_config;
typedef struct omg_mlp_train_config {
    uint32_t epochs;
    uint32_t batch;              /* multiple of 128 */
    float lr, lr_final;          /* cosine decay from lr to lr_final over all steps */
    float weight_decay;          /* AdamW, on weights (not biases) */
    float beta1, beta2, eps;
    uint32_t seed;               /* shuffling */
} omg_mlp_train_config;
int32_t omg_mlp_create(omg_ctx* ctx, const omg_mlp_config* cfg, uint32_t* mlp_id);
int32_t omg_mlp_destroy(omg_ctx* ctx, uint32_t mlp_id);
/* The training set, n rows of n_in inputs and n_out targets (host, row-major). */
int32_t omg_mlp_set_data(omg_ctx* ctx, uint32_t mlp_id, const float* x, const float* y, uint32_t n);
/* Train every member for `epochs` passes over the data; epoch_loss (nullable,
 * members x epochs): the standardized MSE of each epoch's last batch. */
int32_t omg_mlp_train(omg_ctx* ctx, uint32_t mlp_id, const omg_mlp_train_config* cfg, float* epoch_loss);
/* Predict n rows: ensemble mean (and spread, nullable) in the targets' units. */
int32_t omg_surrogate_predict(omg_ctx* ctx, uint32_t mlp_id, const float* x, uint32_t n, float* y_mean,
                              float* y_std);
/* The same, returning per row only the largest ensemble spread among the
 * outputs whose mean is >= level (the usability check of a decay curve) instead
 * of the full spread. */
int32_t omg_surrogate_query(omg_ctx* ctx, uint32_t mlp_id, const float* x, uint32_t n, float* y_mean,
                            float* row_spread, float level);
/* One forward + backward of `member` on standardized x, y (n multiple of 128):
 * the loss and every layer's gradients (W row-major, then b), layer by layer. */
int32_t omg_mlp_grad(omg_ctx* ctx, uint32_t mlp_id, uint32_t member, const float* x, const float* y, uint32_t n,
                     float* loss, float* grads);
/* Checkpoint: what = 1 standardization + weights, 2 AdamW moments + step.
 * out = NULL returns the count only. set_params restores the same layout. */
int32_t omg_mlp_params(omg_ctx* ctx, uint32_t mlp_id, uint32_t what, float* out, uint64_t* count);
int32_t omg_mlp_set_params(omg_ctx* ctx, uint32_t mlp_id, uint32_t what, const float* in, uint64_t count);
/* The tensor-core GEMM alone (tests): C[m x n] = A[m x k] . B[n x k]^T, A and B
 * bf16 bit patterns, row-major with k contiguous; C f32. */
int32_t omg_tc_gemm(omg_ctx* ctx, const uint16_t* a, const uint16_t* b, float* c, uint32_t m, uint32_t n,
                    uint32_t k);
/* Device time of that GEMM at one shape (operands resident, K-major, k a
 * multiple of 8; k_split > 1 splits K over the grid with atomic adds): the
 * mean ms per launch over `reps` launches timed with CUDA events. */
int32_t omg_tc_gemm_bench(omg_ctx* ctx, uint32_t m, uint32_t n, uint32_t k, uint32_t k_split, uint32_t reps,
                          float* ms);

/* ---------------------------------------------------------------- no-alloc */
/* No counterpart in the reference: an addition of this library.
 * omg_trace_box for callers that must not allocate device memory: an audio
 * render callback or other real-time thread (an allocation can block for an
 * unbounded time), or code running while another component owns the device
 * allocator. The caller passes the job, the constants and its own DEVICE
 * output buffers bins_dev[n_bins*n_bands] and dirs_dev[n_bins*3]; the work is
 * queued on cuda_stream (NULL = the legacy default stream) and the call
 * returns without waiting. flags_dev (nullable) is a caller device word that
 * receives the kernels' flag word, as omg_last_flags describes it: 0 when the
 * trace ran to its end, else the trace was cut short (traversal stack, walk
 * budget, params->loop_guard) and the echogram is incomplete; read it after
 * the stream has reached the call. The job is checked as omg_trace_box checks
 * it (finite positions and size, finite materials): OMG_E_INVALID otherwise.
 * The scratch memory lives in one fixed device array per GPU (kept until the
 * process exits), so:
 *  - n_bins * (n_bands + 3) must not exceed OMG_NOALLOC_MAX_CELLS, else
 *    OMG_E_INVALID (about 352 KB of device memory per GPU);
 *  - calls that overlap on the GPU race on that array: order them on one
 *    stream;
 *  - the first call on a device looks up the array's address and loads every
 *    kernel a call may launch (3 or 8 bands, either tie_mode), once per
 *    device, so that no later call waits on the driver's lazy kernel loading;
 *    make it before any stream capture;
 *  - the address is kept for the life of the process: cudaDeviceReset while
 *    this entry point is in use is not supported.
 * It allocates nothing: no cudaMalloc, no cudaFree, no allocating library call. */
#define OMG_NOALLOC_MAX_CELLS 45056   /* 4096 bins x (8 bands + 3) */
int32_t omg_trace_box_noalloc(const omg_box_job* job, const omg_params* params, float* bins_dev, float* dirs_dev,
                              uint32_t* flags_dev, void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* OMG_CUDA_H */
