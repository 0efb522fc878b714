// Shading helpers shared by the persistent kernels (trace.cu) and the
// wavefront kernels (wavefront.cu): compensated histogram adds, the shoebox
// hit, the panel overlay test, the ray-to-job lookup and the shading of a ray
// from its saved state.
#pragma once
#include "device_common.cuh"

namespace omg {

// Compensated accumulation: the atomic returns the old value, so the exact
// rounding error of the add it performed is recovered with TwoSum (Knuth)
// and accumulated in a second float. sum + comp carries ~2x the f32 precision.
// Values are accumulated scaled by 2^64 (kAccScale, exact): float atomics
// flush subnormal operands and results to zero, and a band whose energy has
// decayed below 2^-126 must still add up as the reference's f32 sums do.
__device__ __forceinline__ void acc_add(float* s, float* c, float x) {
  x = x * kAccScale;
  float old = atomicAdd(s, x);
  float sum = old + x;
  float bp = sum - old;
  float err = (old - (sum - bp)) + (x - bp);
  if (err != 0.0f) atomicAdd(c, err);
}

struct Hit {
  float t;
  float nx, ny, nz;
  const DMat* m;
};

// scene.rs:39-88 — analytic shoebox. (Out of line: only shoebox jobs take it,
// and the persistent kernels' loop stays small for the instruction cache.)
static __device__ __noinline__ bool box_hit(const DJob& J, const DMat* __restrict__ job_mats, float px, float py,
                                        float pz, float dx, float dy, float dz, Hit& h) {
  if (!(px > 0.0f && px < J.box[0] && py > 0.0f && py < J.box[1] && pz > 0.0f && pz < J.box[2])) return false;
  float bt = FLT_MAX;
  int bw = 0;
  const float p[3] = {px, py, pz}, d[3] = {dx, dy, dz};
#pragma unroll
  for (int axis = 0; axis < 3; axis++) {
    float di = d[axis];
    if (di > 1e-9f) {
      float t = (J.box[axis] - p[axis]) / di;
      if (t < bt) { bt = t; bw = 2 * axis + 1; }
    } else if (di < -1e-9f) {
      float t = -p[axis] / di;
      if (t < bt) { bt = t; bw = 2 * axis; }
    }
  }
  if (!isfinite(bt) || bt <= 0.0f) return false;
  h.t = bt;
  h.nx = h.ny = h.nz = 0.0f;
  float sgn = (bw % 2 == 0) ? 1.0f : -1.0f;
  int ax = bw / 2;
  if (ax == 0) h.nx = sgn; else if (ax == 1) h.ny = sgn; else h.nz = sgn;
  h.m = job_mats + J.box_mat + bw;
  return true;
}

// scene.rs:94-137 — panel slab ENTRY test, nearest of base and panels.
// Panels are tested group by group: a group (and then a panel) is skipped when
// its box cannot meet the segment's bounding box grown by 1 cm. An entry point
// at t0 in (1e-4, best t) lies on the panel's box and on the segment, so both
// boxes contain it (to within rounding, far below 1 cm at room coordinates).
// Without a base hit the segment is unbounded and every panel is tested. The
// reference scans panels in order with a strict `<`, so among equal entry
// distances the first panel wins: here, the lowest original index.
__device__ __forceinline__ bool panels_hit(const DJob& J, const DPanel* __restrict__ panels,
                                           const DPanelGroup* __restrict__ groups,
                                           const DMat* __restrict__ job_mats, float px, float py, float pz, float dx,
                                           float dy, float dz, bool have, Hit& h) {
  const float p[3] = {px, py, pz}, d[3] = {dx, dy, dz};
  float slo[3], shi[3];
  const bool bounded = have;
  uint32_t best_orig = 0xFFFFFFFFu;  // the current best is the base hit
  if (bounded) {
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const float q = p[a] + d[a] * h.t;
      slo[a] = fminf(p[a], q) - 0.01f;
      shi[a] = fmaxf(p[a], q) + 0.01f;
    }
  }
  for (uint32_t g = 0; g < J.n_groups; g++) {
    const DPanelGroup& G = groups[J.group_off + g];
    if (bounded && (G.mx[0] < slo[0] || G.mn[0] > shi[0] || G.mx[1] < slo[1] || G.mn[1] > shi[1] ||
                    G.mx[2] < slo[2] || G.mn[2] > shi[2]))
      continue;
    for (uint32_t i = G.first; i < G.first + G.count; i++) {
      const DPanel& pn = panels[i];
      if (bounded && (pn.mx[0] < slo[0] || pn.mn[0] > shi[0] || pn.mx[1] < slo[1] || pn.mn[1] > shi[1] ||
                      pn.mx[2] < slo[2] || pn.mn[2] > shi[2]))
        continue;
      float t0 = 0.0f, t1 = FLT_MAX;
      int axis = 3;
      bool miss = false;
#pragma unroll
      for (int a = 0; a < 3; a++) {
        if (miss) break;
        float da = d[a], pa = p[a], lo = pn.mn[a], hi = pn.mx[a];
        if (fabsf(da) < 1e-9f) {
          if (pa < lo || pa > hi) { t0 = FLT_MAX; miss = true; }
        } else {
          float ta = (lo - pa) / da, tb = (hi - pa) / da;
          if (ta > tb) { float tmp = ta; ta = tb; tb = tmp; }
          if (ta > t0) { t0 = ta; axis = a; }
          t1 = fminf(t1, tb);
          if (t0 > t1) { t0 = FLT_MAX; miss = true; }
        }
      }
      const bool closer = !have || t0 < h.t || (t0 == h.t && best_orig != 0xFFFFFFFFu && pn.orig < best_orig);
      if (t0 > 1e-4f && t0 < FLT_MAX && axis < 3 && closer) {
        h.t = t0;
        h.nx = h.ny = h.nz = 0.0f;
        float s = d[axis] > 0.0f ? -1.0f : 1.0f;
        if (axis == 0) h.nx = s; else if (axis == 1) h.ny = s; else h.nz = s;
        h.m = job_mats + pn.mat;
        have = true;
        best_orig = pn.orig;
        if (bounded) {  // the segment only shrinks: tighten its box
#pragma unroll
          for (int a = 0; a < 3; a++) {
            const float q = p[a] + d[a] * h.t;
            slo[a] = fminf(p[a], q) - 0.01f;
            shi[a] = fmaxf(p[a], q) + 0.01f;
          }
        }
      }
    }
  }
  return have;
}

__device__ __forceinline__ uint32_t find_job(const DJob* __restrict__ jobs, uint32_t n_jobs, uint32_t r) {
  uint32_t lo = 0, hi = n_jobs;   // last job with ray_base <= r
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (__ldg(&jobs[mid].ray_base) <= r) lo = mid; else hi = mid;
  }
  return lo;
}


template <int NB>
struct Bands {
  float v[NB];
};

// The receiver sphere's crossing into the compensated histograms: bin `bin`
// gets every band's energy and the direction row -d e_mid (tracer.rs:118-126).
// Out of line: it runs for a few segments in a thousand.
template <int NB>
static __device__ __noinline__ void record_arrival(const DJob& J, float* __restrict__ acc, uint32_t bin, Bands<NB> e,
                                            float dx, float dy, float dz) {
  const uint32_t nb = J.nb;
  float* A = acc + J.acc_off;
  const uint32_t nbb = J.n_bins * nb;
#pragma unroll
  for (int b = 0; b < NB; b++)
    if ((uint32_t)b < nb) acc_add(A + bin * nb + b, A + nbb + bin * nb + b, e.v[b]);
  float em = e.v[0];
#pragma unroll
  for (int b = 1; b < NB; b++)
    if ((uint32_t)b == J.dir_band) em = e.v[b];
  float* D = A + 2 * nbb;
  const uint32_t nd = J.n_bins * 3;
  acc_add(D + bin * 3 + 0, D + nd + bin * 3 + 0, -(dx * em));
  acc_add(D + bin * 3 + 1, D + nd + bin * 3 + 1, -(dy * em));
  acc_add(D + bin * 3 + 2, D + nd + bin * 3 + 2, -(dz * em));
}

// One segment after its closest hit (tracer.rs:110-200): the receiver test with
// compensated histogram adds, then advance, absorb, transmit or scatter.
// Returns true when the ray ends here.
template <int NB>
__device__ __forceinline__ bool shade_segment(const DJob& J, float* __restrict__ acc, const Hit& h, bool have,
                                              float t_hit, float& px, float& py, float& pz, float& dx, float& dy,
                                              float& dz, float& dist, float (&e)[NB], Pcg& rng) {
  const uint32_t nb = J.nb;
  // receiver sphere crossing along this segment (tracer.rs:110-128)
  {
    const float tlx = J.lis[0] - px, tly = J.lis[1] - py, tlz = J.lis[2] - pz;
    const float s = tlx * dx + tly * dy + tlz * dz;
    if (s > 0.0f && s < t_hit) {
      const float cx = px + dx * s, cy = py + dy * s, cz = pz + dz * s;
      const float ddx = cx - J.lis[0], ddy = cy - J.lis[1], ddz = cz - J.lis[2];
      if (sqrtf(ddx * ddx + ddy * ddy + ddz * ddz) < J.rr) {
        const float arrival = (dist + s) / J.c;
        const float q = arrival / J.bin_dt;
        if (q < (float)J.n_bins) {          // (q as usize) < NBINS, q >= 0
          Bands<NB> eb;
#pragma unroll
          for (int b = 0; b < NB; b++) eb.v[b] = e[b];
          record_arrival<NB>(J, acc, (uint32_t)q, eb, dx, dy, dz);
        }
      }
    }
  }

  bool done = !have;
  if (!done) {
    px = px + dx * t_hit;
    py = py + dy * t_hit;
    pz = pz + dz * t_hit;
    dist = dist + t_hit;
    if (dist / J.c > J.max_time) done = true;
  }
  if (!done) {
    const DMat& M = *h.m;
    const float p = M.p;
    bool alive = false;
    if (p > 0.0f && rng.f32() < p) {
      // through-the-wall branch (tracer.rs:160-173)
#pragma unroll
      for (int b = 0; b < NB; b++)
        if ((uint32_t)b < nb) {
          e[b] = e[b] * M.wt[b];
          if (e[b] > J.floor_e) alive = true;
        }
      if (!alive) {
        done = true;
      } else {
        const float step = 2.0f * J.wall_eps;
        px = px + dx * step;
        py = py + dy * step;
        pz = pz + dz * step;
      }
    } else {
#pragma unroll
      for (int b = 0; b < NB; b++)
        if ((uint32_t)b < nb) {
          e[b] = e[b] * M.wr[b];
          if (e[b] > J.floor_e) alive = true;
        }
      if (!alive) {
        done = true;
      } else {
        const float nx = h.nx, ny = h.ny, nz = h.nz;
        if (rng.f32() < M.scattering) {
          float ux, uy, uz;
          unit_sphere(rng, ux, uy, uz);
          float ax = nx + ux, ay = ny + uy, az = nz + uz;
          normalize3(ax, ay, az);
          if (ax * nx + ay * ny + az * nz < 1e-3f) { ax = nx; ay = ny; az = nz; }
          dx = ax; dy = ay; dz = az;
        } else {
          const float k = 2.0f * (dx * nx + dy * ny + dz * nz);
          dx = dx - nx * k;
          dy = dy - ny * k;
          dz = dz - nz * k;
        }
        px = px + nx * J.wall_eps;
        py = py + ny * J.wall_eps;
        pz = pz + nz * J.wall_eps;
      }
    }
  }
  return done;
}

// One segment of ray r from its saved state (WfState records): the closest
// hit (a mesh hit saved by the walk, or the analytic shoebox), the panels,
// then shade_segment. A surviving ray's state is stored back and true is
// returned; a finished ray adds its segment count to its job.
template <int NB>
__device__ __forceinline__ bool shade_saved_ray(const DJob* __restrict__ jobs, uint32_t n_jobs,
                                                const DScene* __restrict__ scenes,
                                                const DMat* __restrict__ job_mats,
                                                const DPanel* __restrict__ panels,
                                                const DPanelGroup* __restrict__ groups, float* __restrict__ acc,
                                                const WfState& st, uint32_t r,
                                                uint32_t* __restrict__ job_segments) {
  const uint32_t ji = find_job(jobs, n_jobs, r);
  const DJob& J = jobs[ji];
  const float4 P = st.pos[r], D = st.dir[r];
  float px = P.x, py = P.y, pz = P.z, dist = P.w;
  float dx = D.x, dy = D.y, dz = D.z;
  Pcg rng;
  rng.s = __float_as_uint(D.w);
  float e[NB];
  {
    const float4 e0 = st.e[r];
    const float4 e1 = NB > 4 ? st.e[st.cap + r] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float ev[8] = {e0.x, e0.y, e0.z, e0.w, e1.x, e1.y, e1.z, e1.w};
#pragma unroll
    for (int b = 0; b < NB; b++) e[b] = ev[b];
  }
  uint32_t bounce = st.bounce[r];
  Hit h;
  h.t = FLT_MAX;
  h.m = nullptr;
  bool have;
  if (J.geom == OMG_GEOM_BOX) {
    have = box_hit(J, job_mats, px, py, pz, dx, dy, dz, h);
  } else {
    const float2 H = st.hit[r];
    const int prim = __float_as_int(H.y);
    have = prim >= 0;
    if (have) {
      const DScene& S = scenes[J.scene];
      const float4 p0 = __ldg(S.prims + 3 * prim + 0);
      const float4 p1 = __ldg(S.prims + 3 * prim + 1);
      const float4 nn = __ldg(S.normals + __float_as_uint(p1.w));
      float nx = nn.x, ny = nn.y, nz = nn.z;
      if (nx * dx + ny * dy + nz * dz > 0.0f) { nx = nx * -1.0f; ny = ny * -1.0f; nz = nz * -1.0f; }
      h.t = H.x;
      h.nx = nx; h.ny = ny; h.nz = nz;
      h.m = S.mats + __float_as_uint(p0.w);
    }
  }
  if (J.n_groups) have = panels_hit(J, panels, groups, job_mats, px, py, pz, dx, dy, dz, have, h);
  const float t_hit = have ? h.t : FLT_MAX;
  bool done = shade_segment<NB>(J, acc, h, have, t_hit, px, py, pz, dx, dy, dz, dist, e, rng);
  bounce++;
  if (!done && bounce >= J.max_bounces) done = true;
  if (done) {
    atomicAdd(job_segments + ji, bounce);
    return false;
  }
  st.pos[r] = make_float4(px, py, pz, dist);
  st.dir[r] = make_float4(dx, dy, dz, __uint_as_float(rng.s));
  float v[8];
#pragma unroll
  for (int b = 0; b < 8; b++) v[b] = b < NB ? e[b] : 0.0f;
  st.e[r] = make_float4(v[0], v[1], v[2], v[3]);
  if (NB > 4) st.e[st.cap + r] = make_float4(v[4], v[5], v[6], v[7]);
  st.bounce[r] = bounce;
  return true;
}

// A fresh ray's saved state (tracer.rs:96-102): stream, direction, source,
// energies, no segment yet.
template <int NB>
__device__ __forceinline__ void start_saved_ray(const DJob& J, const WfState& st, uint32_t r) {
  Pcg rng;
  rng.init(J.seed, r - J.ray_base);
  float dx, dy, dz;
  unit_sphere(rng, dx, dy, dz);
  st.pos[r] = make_float4(J.src[0], J.src[1], J.src[2], 0.0f);
  st.dir[r] = make_float4(dx, dy, dz, __uint_as_float(rng.s));
  float v[8];
#pragma unroll
  for (int b = 0; b < 8; b++) v[b] = b < NB ? J.e0[b] : 0.0f;
  st.e[r] = make_float4(v[0], v[1], v[2], v[3]);
  if (NB > 4) st.e[st.cap + r] = make_float4(v[4], v[5], v[6], v[7]);
  st.bounce[r] = 0;
}

}  // namespace omg
