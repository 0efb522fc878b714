// Ambient-dome fan on the GPU (crates/omg-scene/src/dome.rs:293-478).
//
// One thread per (listener, fan ray): the specular escape (trace_escape,
// dome.rs:330-382: <= max_events mesh hits or pane crossings, 80 m horizon)
// and, when the escape is not near-full, the straight-through mass-law seep
// (trace_through, dome.rs:390-422, over segment_hits, mesh.rs:546-604). A
// second kernel bins the rays of each listener in fan order (dome.rs:452-458,
// the same f32 sums in the same order), applies the per-listener EMA and
// writes the 9 bins. The fan is deterministic, so the result is too.
#include "device_common.cuh"

namespace omg {

namespace {

constexpr float PI_F = 3.14159265358979323846f;
constexpr uint32_t kMaxCross = 64;   // crossings kept per straight-through segment

// dome.rs:56-68
__device__ __forceinline__ bool panel_hit(const DDomePanel& p, float ox, float oy, float oz, float dx, float dy,
                                          float dz, float t_max, float& tout) {
  const float po = p.axis == 0 ? ox : oy, pd = p.axis == 0 ? dx : dy;
  if (fabsf(pd) < 1e-8f) return false;
  const float t = (p.plane - po) / pd;
  if (t < 1e-4f || t >= t_max) return false;
  const float lat = p.axis == 0 ? oy + t * dy : ox + t * dx;
  const float z = oz + t * dz;
  if (lat > p.lat0 && lat < p.lat1 && z > p.z0 && z < p.z1) {
    tout = t;
    return true;
  }
  return false;
}

// dome.rs:328-382. Returns true (escaped) with the throughput in tp.
template <bool TIE>
__device__ bool trace_escape(const DScene& S, const DDomeLaunch& L, float px, float py, float pz, float dx, float dy,
                             float dz, float tp[MAXB], uint32_t& events) {
  const uint32_t nb = L.nb;
#pragma unroll
  for (int b = 0; b < MAXB; b++) tp[b] = 1.0f;
  for (uint32_t ev = 0; ev < L.max_events; ev++) {
    events++;
    float tm = FLT_MAX;
    int prim = 0;
    const bool mh = mesh_closest<TIE>(S, px, py, pz, dx, dy, dz, tm, prim, &L.hdr->error);
    const float t_mesh = mh ? tm : FLT_MAX;
    float t_pan = t_mesh;
    int pan = -1;
    for (uint32_t k = 0; k < L.n_panels; k++) {
      float t;
      if (panel_hit(L.panels[k], px, py, pz, dx, dy, dz, t_pan, t)) {
        t_pan = t;
        pan = (int)k;
      }
    }
    if (pan >= 0) {
      const DDomePanel& P = L.panels[pan];
      if (!P.glass) return false;  // a door leaf blocks
#pragma unroll
      for (int b = 0; b < MAXB; b++)
        if ((uint32_t)b < nb) tp[b] = tp[b] * P.t2[b];
      const float adv = t_pan + 1e-3f;
      px = px + dx * adv;
      py = py + dy * adv;
      pz = pz + dz * adv;
      continue;
    }
    const bool escaped = pz > -0.05f || dz > 0.05f;
    if (!mh) return escaped;
    if (tm > 80.0f) return escaped;
    const float4 p0 = __ldg(S.prims + 3 * prim);
    const float4 p1 = __ldg(S.prims + 3 * prim + 1);
    const DMat& M = S.mats[__float_as_uint(p0.w)];
#pragma unroll
    for (int b = 0; b < MAXB; b++)
      if ((uint32_t)b < nb) tp[b] = tp[b] * (1.0f - M.absorption[b]);
    if (tp[1] < 2e-3f) return false;
    const float4 nn = __ldg(S.normals + __float_as_uint(p1.w));
    const float nx = nn.x, ny = nn.y, nz = nn.z;
    const float dn = dx * nx + dy * ny + dz * nz;
    float ox = nx, oy = ny, oz = nz;
    if (dn > 0.0f) { ox = nx * -1.0f; oy = ny * -1.0f; oz = nz * -1.0f; }
    const float hx = px + dx * tm, hy = py + dy * tm, hz = pz + dz * tm;
    const float k2 = 2.0f * dn;
    dx = dx - nx * k2;
    dy = dy - ny * k2;
    dz = dz - nz * k2;
    normalize3(dx, dy, dz);
    px = hx + ox * 1e-3f;
    py = hy + oy * 1e-3f;
    pz = hz + oz * 1e-3f;
  }
  return false;
}

struct Cross {
  float t;
  uint32_t tri;
  uint32_t mat;
};

// mesh.rs:546-604: every crossing strictly inside a->b, in the reference's
// visit order (right subtree first), stably sorted, same-t clusters merged to
// the lowest surface id. Returns the count (kMaxCross + 1 = overflow).
__device__ uint32_t segment_hits(const DScene& S, float ax, float ay, float az, float bx, float by, float bz,
                                 Cross* out) {
  if (S.n_prims == 0) return 0;
  float dx = bx - ax, dy = by - ay, dz = bz - az;
  const float len = sqrtf(dx * dx + dy * dy + dz * dz);
  if (len < 1e-6f) return 0;
  const float il = __frcp_rn(len);
  dx = dx * il;
  dy = dy * il;
  dz = dz * il;
  const float ix = __frcp_rn(dx), iy = __frcp_rn(dy), iz = __frcp_rn(dz);
  uint32_t n = 0;
  bool overflow = false;
  int stack[STACK_DEPTH];
  int sp = 0;
  stack[sp++] = S.root;
  while (sp > 0) {
    const int cur = stack[--sp];
    if (cur >= 0) {
      const float4 n0 = __ldg(S.nodes + 4 * cur + 0);
      const float4 n1 = __ldg(S.nodes + 4 * cur + 1);
      const float4 n2 = __ldg(S.nodes + 4 * cur + 2);
      const float4 n3 = __ldg(S.nodes + 4 * cur + 3);
      float ta, tb;
      const bool h0 = ray_aabb(n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, ax, ay, az, ix, iy, iz, len, ta);
      const bool h1 = ray_aabb(n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, ax, ay, az, ix, iy, iz, len, tb);
      // the reference pushes left then right and pops right first
      if (h0) {
        if (sp < STACK_DEPTH) stack[sp++] = __float_as_int(n3.x);
        else overflow = true;
      }
      if (h1) {
        if (sp < STACK_DEPTH) stack[sp++] = __float_as_int(n3.y);
        else overflow = true;
      }
    } else {
      const uint32_t code = ~(uint32_t)cur;
      const uint32_t start = code >> 3, end = start + (code & 7u) + 1u;
      for (uint32_t i = start; i < end; i++) {
        const float4 p0 = __ldg(S.prims + 3 * i + 0);
        const float4 p1 = __ldg(S.prims + 3 * i + 1);
        const float4 p2 = __ldg(S.prims + 3 * i + 2);
        float t;
        if (ray_tri(p0, p1, p2, ax, ay, az, dx, dy, dz, t)) {
          const float tt = t / len;
          if (tt > 1e-4f && tt < 1.0f - 1e-4f) {
            if (n < kMaxCross) out[n++] = Cross{tt, __float_as_uint(p1.w), __float_as_uint(p0.w)};
            else overflow = true;
          }
        }
      }
    }
  }
  if (overflow) return kMaxCross + 1;
  // stable insertion sort by t
  for (uint32_t i = 1; i < n; i++) {
    const Cross c = out[i];
    uint32_t j = i;
    while (j > 0 && out[j - 1].t > c.t) {
      out[j] = out[j - 1];
      j--;
    }
    out[j] = c;
  }
  const float tol = 1e-4f / fmaxf(len, 1.0f);
  uint32_t w = 0;
  for (uint32_t i = 0; i < n; i++) {
    if (w > 0 && fabsf(out[i].t - out[w - 1].t) < tol) {
      if (S.tri_surface[out[i].tri] < S.tri_surface[out[w - 1].tri]) {
        out[w - 1].tri = out[i].tri;
        out[w - 1].mat = out[i].mat;
      }
    } else {
      out[w++] = out[i];
    }
  }
  return w;
}

// dome.rs:384-422
__device__ void trace_through(const DScene& S, const DDomeLaunch& L, float ex, float ey, float ez, float dx,
                              float dy, float dz, float tp[MAXB]) {
  const uint32_t nb = L.nb;
  const float bx = ex + dx * 50.0f, by = ey + dy * 50.0f, bz = ez + dz * 50.0f;
#pragma unroll
  for (int b = 0; b < MAXB; b++) tp[b] = 1.0f;
  if (bz < -0.05f) {
#pragma unroll
    for (int b = 0; b < MAXB; b++) tp[b] = 0.0f;
    return;
  }
  Cross hits[kMaxCross];
  const uint32_t nh = segment_hits(S, ex, ey, ez, bx, by, bz, hits);
  if (nh > kMaxCross) {
    atomicOr(&L.hdr->error, 2u);
#pragma unroll
    for (int b = 0; b < MAXB; b++) tp[b] = 0.0f;
    return;
  }
  for (uint32_t h = 0; h < nh; h++) {
    const DMat& M = S.mats[hits[h].mat];
#pragma unroll
    for (int b = 0; b < MAXB; b++)
      if ((uint32_t)b < nb) tp[b] = tp[b] * M.t2[b];
    if (tp[0] < 1e-7f) {
#pragma unroll
      for (int b = 0; b < MAXB; b++) tp[b] = 0.0f;
      return;
    }
  }
  for (uint32_t k = 0; k < L.n_panels; k++) {
    float t;
    if (panel_hit(L.panels[k], ex, ey, ez, dx, dy, dz, 80.0f, t)) {
#pragma unroll
      for (int b = 0; b < MAXB; b++)
        if ((uint32_t)b < nb) tp[b] = tp[b] * L.panels[k].t2[b];
    }
  }
}

template <bool TIE>
__global__ void dome_rays_kernel(DDomeLaunch L) {
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= L.n_eyes * L.n_rays) return;
  const uint32_t eye = gid / L.n_rays, j = gid % L.n_rays;
  const DScene S = *L.scene;
  const uint32_t i = (uint32_t)((uint64_t)j * L.n_fan / L.n_rays);  // dome.rs:434
  const float4 f = L.fan[i];
  const float ex = L.eyes[3 * eye], ey = L.eyes[3 * eye + 1], ez = L.eyes[3 * eye + 2];
  float bp[MAXB], tp[MAXB];
  uint32_t events = 0, through = 0;
  const bool esc = trace_escape<TIE>(S, L, ex, ey, ez, f.x, f.y, f.z, bp, events);
  if (esc && bp[0] > 0.5f) {
#pragma unroll
    for (int b = 0; b < MAXB; b++) tp[b] = bp[b];
  } else {
    through = 1;
    trace_through(S, L, ex, ey, ez, f.x, f.y, f.z, tp);
    if (esc) {
#pragma unroll
      for (int b = 0; b < MAXB; b++) tp[b] = fmaxf(tp[b], bp[b]);
    }
  }
  float* o = L.ray_tp + (uint64_t)gid * L.nb;
  for (uint32_t b = 0; b < L.nb; b++) o[b] = tp[b];
  L.ray_escape[gid] = esc ? 1 : 0;
  atomicAdd(&L.events[0], events);
  if (through) atomicAdd(&L.events[1], through);
}

// dome.rs:452-477 per listener: bins in fan order, EMA, directions.
__global__ void dome_bins_kernel(DDomeLaunch L, float ema_alpha) {
  const uint32_t eye = blockIdx.x;
  const uint32_t k = threadIdx.x;  // bin 0..8; lanes 9..31 only join the warp sync
  const uint32_t nb = L.nb;
  const bool primed = L.primed[eye] != 0u;
  __syncwarp();
  if (k < 9) {
    float e[MAXB];
#pragma unroll
    for (int b = 0; b < MAXB; b++) e[b] = 0.0f;
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    const float nr = (float)L.n_rays;
    for (uint32_t j = 0; j < L.n_rays; j++) {
      const uint32_t i = (uint32_t)((uint64_t)j * L.n_fan / L.n_rays);
      const float4 f = L.fan[i];
      if ((uint32_t)__float_as_int(f.w) != k) continue;
      const float* tp = L.ray_tp + ((uint64_t)eye * L.n_rays + j) * nb;
      if (tp[0] > 1e-9f) {
#pragma unroll
        for (int b = 0; b < MAXB; b++)
          if ((uint32_t)b < nb) e[b] = e[b] + tp[b] / nr;
        const float w = fmaxf(tp[1], tp[0] * 0.2f);
        sx = sx + f.x * w;
        sy = sy + f.y * w;
        sz = sz + f.z * w;
      }
    }
    const float alpha = primed ? ema_alpha : 1.0f;
    float* ema = L.ema + ((uint64_t)eye * 9 + k) * nb;
    for (uint32_t b = 0; b < nb; b++) {
      L.raw[((uint64_t)eye * 9 + k) * nb + b] = e[b];
      ema[b] = ema[b] + alpha * (e[b] - ema[b]);
      L.out_energy[((uint64_t)eye * 9 + k) * nb + b] = ema[b];
    }
    float dxo, dyo, dzo;
    if (sqrtf(sx * sx + sy * sy + sz * sz) > 1e-6f) {
      dxo = sx; dyo = sy; dzo = sz;
      normalize3(dxo, dyo, dzo);
    } else if (k == 8) {
      dxo = 0.0f; dyo = 0.0f; dzo = 1.0f;
    } else {
      const float az = ((float)k + 0.5f) * TAU_F / 8.0f - PI_F;
      double s, c;
      sincos((double)az, &s, &c);
      dxo = (float)c; dyo = (float)s; dzo = 0.0f;
    }
    float* od = L.out_dir + ((uint64_t)eye * 9 + k) * 3;
    od[0] = dxo;
    od[1] = dyo;
    od[2] = dzo;
  }
  __syncwarp();
  if (k == 0) L.primed[eye] = 1u;
}

// dome.rs:316-324 fan + dome.rs:304-310 bin per direction (in .w)
__global__ void fan_kernel(float4* fan, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float ga = PI_F * (3.0f - sqrtf(5.0f));
  const float z = 1.0f - 2.0f * ((float)i + 0.5f) / (float)n;
  const float r = sqrtf(fmaxf(1.0f - z * z, 0.0f));
  const float phi = ga * (float)i;
  double s, c;
  sincos((double)phi, &s, &c);
  const float x = r * (float)c, y = r * (float)s;
  int bin;
  if (z > 0.87f) {
    bin = 8;
  } else {
    const float az = (float)atan2((double)y, (double)x) + PI_F;
    const float q = az / (TAU_F / 8.0f);
    uint32_t b = q >= 0.0f ? (uint32_t)q : 0u;
    bin = (int)(b < 7u ? b : 7u);
  }
  fan[i] = make_float4(x, y, z, __int_as_float(bin));
}

}  // namespace

cudaError_t build_dome_fan(float4* fan, uint32_t n, cudaStream_t s) {
  fan_kernel<<<(n + 127) / 128, 128, 0, s>>>(fan, n);
  return cudaGetLastError();
}

cudaError_t launch_dome(const DDomeLaunch& L, cudaStream_t s) {
  const uint64_t total = (uint64_t)L.n_eyes * L.n_rays;
  if (total == 0) return cudaSuccess;
  if (L.tie) dome_rays_kernel<true><<<(uint32_t)((total + 127) / 128), 128, 0, s>>>(L);
  else dome_rays_kernel<false><<<(uint32_t)((total + 127) / 128), 128, 0, s>>>(L);
  dome_bins_kernel<<<L.n_eyes, 32, 0, s>>>(L, 0.35f);
  return cudaGetLastError();
}

}  // namespace omg
