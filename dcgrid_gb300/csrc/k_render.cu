// k_render.cu — headless volume ray marcher.
//
// Restates the reference's renderer (src/raymarching.cuh:17-275, samplers of
// src/dcgrid/dcgrid_rendering.cu:6-56 and src/uniformgrid/
// uniformgrid_rendering.cu:5-52, camera of k_dcgrid_render,
// dcgrid_rendering.cu:58-92) as one CUDA kernel that writes RGBA float4 per
// pixel into a device buffer instead of a GL surface: per pixel and
// antialiasing sample, a ray from the eye marches the domain box with steps of
// at least half a cell, composites the density with front-to-back alpha,
// optionally marches toward the sun for shadows, and shades the floor, the
// scene SDF and the debug slice channels.
#include "dcg_dev.cuh"
#include "dcg_kernels.h"

namespace dcg {

namespace {

struct F3 {
  float x, y, z;
};
__device__ inline F3 f3(float x, float y, float z) { return {x, y, z}; }
__device__ inline F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ inline F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ inline F3 operator*(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ inline F3 operator/(F3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ inline float dot3(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ inline float len3(F3 a) { return sqrtf(dot3(a, a)); }
__device__ inline F3 normalize3(F3 a) { return a * (1.f / len3(a)); }
__device__ inline F3 inv3(F3 a) { return {1.f / a.x, 1.f / a.y, 1.f / a.z}; }

// colors.cuh mix: front-to-back compositing of (src, srcAlpha) under (dst, dstAlpha)
__device__ inline void mix(F3 src, float srcAlpha, F3 &dst, float &dstAlpha) {
  if (srcAlpha > 1e-6f) {
    const float impact = (1.f - dstAlpha) * srcAlpha;
    dst = (dst * dstAlpha + src * impact) / (dstAlpha + impact);
    dstAlpha += impact;
  }
}

struct March {  // MarchAux (raymarching.cuh:19-43)
  int ix, iy, iz;
  float fx, fy, fz;
  size_t idx[8];
  int scale;
  float density;
};

template <class Field> __device__ inline float interp(const March &a, Field f) {
  const float dxInv = 1.f - a.fx;
  const float c00 = f(a.idx[0]) * dxInv + f(a.idx[4]) * a.fx;
  const float c01 = f(a.idx[1]) * dxInv + f(a.idx[5]) * a.fx;
  const float c10 = f(a.idx[2]) * dxInv + f(a.idx[6]) * a.fx;
  const float c11 = f(a.idx[3]) * dxInv + f(a.idx[7]) * a.fx;
  const float dyInv = 1.f - a.fy;
  const float c0 = c00 * dyInv + c10 * a.fy;
  const float c1 = c01 * dyInv + c11 * a.fy;
  return c0 * (1.f - a.fz) + c1 * a.fz;
}

// Adaptive grid samplers (dcgrid_rendering.cu:6-56): the finest block over the
// sample, then either its nearest cell or a trilinear read of its apron.
struct AdaptiveGrid {
  const Dev &D;
  __device__ float q(size_t i) const { return q_ld(D, 0, i); }
  __device__ const Geom &g() const { return D.g; }
  __device__ const Phys &ph() const { return D.ph; }
  __device__ float vel_len(const March &a) const {
    const float vx = interp(a, [&](size_t i) { return D.v[0][i]; });
    const float vy = interp(a, [&](size_t i) { return D.v[1][i]; });
    const float vz = interp(a, [&](size_t i) { return D.v[2][i]; });
    return sqrtf(vx * vx + vy * vy + vz * vz);
  }
  __device__ float fluid(const March &a) const {
    return interp(a, [&](size_t i) { return D.w[i]; });
  }
  __device__ void sample(F3 p, bool precise, March &a) const {
    a.ix = clampi((int)floorf(p.x), 0, D.g.gx - 1);
    a.iy = clampi((int)floorf(p.y), 0, D.g.gy - 1);
    a.iz = clampi((int)floorf(p.z), 0, D.g.gz - 1);
    int lev;
    const uint32_t b = locate(D, a.ix, a.iy, a.iz, 0, lev);
    const int4 bp = D.pos[b];
    a.scale = 1 << lev;
    if (!precise) {
      // the reference indexes the block with the finest cell's coordinates
      // mod 4 at every level (dcgrid_rendering.cu:11-14); ref_compat = 0 uses
      // the cell of the block's own level
      const int sh = D.g.ref_compat ? 0 : lev;
      const size_t c = (size_t)b * BV + local_of((a.ix >> sh) & 3, (a.iy >> sh) & 3, (a.iz >> sh) & 3);
      for (int k = 0; k < 8; k++) a.idx[k] = c;
      a.fx = a.fy = a.fz = 0.f;
      a.density = q(c);
      return;
    }
    const float si = 1.f / (float)a.scale;
    const float x = p.x * si - .5f, y = p.y * si - .5f, z = p.z * si - .5f;
    const float xf = floorf(x), yf = floorf(y), zf = floorf(z);
    a.fx = x - xf;
    a.fy = y - yf;
    a.fz = z - zf;
    const int i = (int)xf + 1 - bp.x, j = (int)yf + 1 - bp.y, k = (int)zf + 1 - bp.z;
    a.idx[0] = apron_cell(D, b, bp, i, j, k);
    a.idx[1] = apron_cell(D, b, bp, i, j, k + 1);
    a.idx[2] = apron_cell(D, b, bp, i, j + 1, k);
    a.idx[3] = apron_cell(D, b, bp, i, j + 1, k + 1);
    a.idx[4] = apron_cell(D, b, bp, i + 1, j, k);
    a.idx[5] = apron_cell(D, b, bp, i + 1, j, k + 1);
    a.idx[6] = apron_cell(D, b, bp, i + 1, j + 1, k);
    a.idx[7] = apron_cell(D, b, bp, i + 1, j + 1, k + 1);
    a.density = interp(a, [&](size_t c) { return q(c); });
  }
};

// Uniform grid samplers (uniformgrid_rendering.cu:5-52)
struct UniformGridR {
  const UDev &U;
  __device__ const Geom &g() const { return U.g; }
  __device__ const Phys &ph() const { return U.ph; }
  __device__ float vel_len(const March &a) const {
    const float vx = interp(a, [&](size_t i) { return U.v[0][i]; });
    const float vy = interp(a, [&](size_t i) { return U.v[1][i]; });
    const float vz = interp(a, [&](size_t i) { return U.v[2][i]; });
    return sqrtf(vx * vx + vy * vy + vz * vz);
  }
  __device__ float fluid(const March &a) const {
    return interp(a, [&](size_t i) { return U.w[i]; });
  }
  __device__ size_t at(int x, int y, int z) const { return ((size_t)z * U.gy + y) * U.gx + x; }
  __device__ void sample(F3 p, bool precise, March &a) const {
    a.scale = 1;
    if (!precise) {
      a.ix = clampi((int)p.x, 0, U.gx - 1);
      a.iy = clampi((int)p.y, 0, U.gy - 1);
      a.iz = clampi((int)p.z, 0, U.gz - 1);
      const size_t c = at(a.ix, a.iy, a.iz);
      for (int k = 0; k < 8; k++) a.idx[k] = c;
      a.fx = a.fy = a.fz = 0.f;
      a.density = U.q[0][c];
      return;
    }
    const float x = p.x - .5f, y = p.y - .5f, z = p.z - .5f;
    const float xf = floorf(x), yf = floorf(y), zf = floorf(z);
    a.ix = (int)xf; a.iy = (int)yf; a.iz = (int)zf;
    a.fx = x - xf; a.fy = y - yf; a.fz = z - zf;
    const int x0 = clampi(a.ix, 0, U.gx - 1), y0 = clampi(a.iy, 0, U.gy - 1), z0 = clampi(a.iz, 0, U.gz - 1);
    const size_t xs = a.ix < U.gx - 1 ? 1 : 0, ys = a.iy < U.gy - 1 ? (size_t)U.gx : 0,
                 zs = a.iz < U.gz - 1 ? (size_t)U.gx * U.gy : 0;
    a.idx[0] = at(x0, y0, z0);
    a.idx[1] = a.idx[0] + zs;
    a.idx[2] = a.idx[0] + ys;
    a.idx[3] = a.idx[1] + ys;
    a.idx[4] = a.idx[0] + xs;
    a.idx[5] = a.idx[4] + zs;
    a.idx[6] = a.idx[4] + ys;
    a.idx[7] = a.idx[6] + zs;
    a.density = interp(a, [&](size_t c) { return U.q[0][c]; });
  }
};

__device__ inline float sdf(const Geom &g, const Phys &ph, F3 p) { return scene_sdf(g, ph, p.x, p.y, p.z); }

// estimateNormal (sdf.cuh:25-34)
__device__ inline F3 sdf_normal(const Geom &g, const Phys &ph, F3 p) {
  const float e = 1e-4f;
  return normalize3(f3(sdf(g, ph, f3(p.x + e, p.y, p.z)) - sdf(g, ph, f3(p.x - e, p.y, p.z)),
                       sdf(g, ph, f3(p.x, p.y + e, p.z)) - sdf(g, ph, f3(p.x, p.y - e, p.z)),
                       sdf(g, ph, f3(p.x, p.y, p.z + e)) - sdf(g, ph, f3(p.x, p.y, p.z - e))));
}

// rayDomainIntersections (raymarching.cuh:52-78)
__device__ inline bool box_hit(const Geom &g, float &dNear, float &dFar, F3 o, F3 dinv) {
  const float cx = g.gx * .5f, cy = g.gy * .5f, cz = g.gz * .5f;
  const float nx = dinv.x * (o.x - cx), ny = dinv.y * (o.y - cy), nz = dinv.z * (o.z - cz);
  const float kx = fabsf(dinv.x) * cx, ky = fabsf(dinv.y) * cy, kz = fabsf(dinv.z) * cz;
  dNear = fmaxf(fmaxf(-nx - kx, -ny - ky), -nz - kz);
  dFar = fminf(fminf(-nx + kx, -ny + ky), -nz + kz);
  return dNear < dFar && dFar > 0.f;
}

__device__ inline float density_alpha(float dx, float dist, float dens) { return 1.f - expf(-dist * dx * dens); }

enum { CH_FLUID = 0, CH_DENSITY = 1, CH_VELOCITY = 2, CH_FLUIDITY = 3, CH_RESOLUTION = 4 };

// lightmarch (raymarching.cuh:80-117)
template <class Grid>
__device__ float light_march(const Grid &G, const RenderP &R, F3 origin, F3 sun, F3 suninv) {
  float light = 1.f;
  const Geom &g = G.g();
  const Phys &ph = G.ph();
  if (R.solids && ph.solids) {
    float dScene = 0.f;
    for (int i = 0; i < 100; i++) {
      const float s = sdf(g, ph, origin + sun * dScene);
      light = fminf(light, (s / dScene) / .06f);
      if (light <= 1e-2f) return 0.f;
      dScene += s;
    }
  }
  if (R.channel == CH_FLUID) {
    float dNear, dFar;
    if (box_hit(g, dNear, dFar, origin, suninv)) {
      F3 pos = origin;
      if (dNear > 0.f) {
        pos = pos + sun * dNear;
        dFar -= dNear;
      }
      const float step = fmaxf(dFar / 100.f, 1e-1f);
      float dens = 0.f;
      March a;
      for (float d = step; d < dFar && dens < 5.f; d += step) {
        pos = pos + sun * step;
        G.sample(pos, R.precise != 0, a);
        dens += a.density * ph.dx * step;
      }
      light *= expf(-dens);
    }
  }
  return light;
}

// raymarch (raymarching.cuh:119-271)
template <class Grid>
__device__ float4 ray_march(const Grid &G, const RenderP &R, F3 origin, F3 dir, F3 sun) {
  const Geom &g = G.g();
  const Phys &ph = G.ph();
  const float ambInv = 1.f - R.ambient;
  const float floorLight = fmaxf(0.f, sun.y);
  const float sliceZ = g.gz * .5f;
  const F3 dinv = inv3(dir), suninv = inv3(sun);
  const F3 smoke = f3(R.smoke[0], R.smoke[1], R.smoke[2]);
  float dCurrent = 0.f, dSolid = 3.402823466e+38f, light;
  F3 color = f3(0.f, 0.f, 0.f);
  float alpha = 0.f;
  int what = 0;  // 1 scene, 2 floor, 3 debug slice
  if (R.channel != CH_FLUID && (sliceZ - origin.z) * dir.z > 0.f) {
    const float d = (sliceZ - origin.z) / dir.z;
    const float px = origin.x + d * dir.x, py = origin.y + d * dir.y;
    if (px >= 0.f && py >= 0.f && px < g.gx && py < g.gy && d < dSolid) {
      dSolid = d;
      what = 3;
    }
  }
  if (R.solids && (0.f - origin.y) * dir.y > 0.f) {
    const float d = (0.f - origin.y) / dir.y;
    if (d < dSolid) {
      dSolid = d;
      what = 2;
    }
  }
  if (R.solids && ph.solids) {
    float s = 3.402823466e+38f, dScene = dCurrent;
    for (int i = 0; i < 100; i++) {
      s = sdf(g, ph, origin + dir * dScene);
      if (s < 1e-1f || dScene >= dSolid) break;
      dScene += s;
    }
    if (s < 1e-1f && dScene < dSolid) {
      dSolid = dScene;
      what = 1;
    }
  }
  March a;
  if (R.channel == CH_FLUID) {
    float dNear, dFar;
    if (box_hit(g, dNear, dFar, origin, dinv)) {
      dCurrent = fmaxf(dCurrent, fmaxf(dNear, 10.f));
      F3 pos = origin + dir * dCurrent;
      const float dMax = fminf(dFar, dSolid);
      while (dCurrent < dMax && alpha <= .99f) {
        const F3 prev = pos;
        dCurrent = fminf(fmaxf(dCurrent * 1.f, dCurrent + .5f), dMax);
        pos = origin + dir * dCurrent;
        G.sample((prev + pos) * .5f, R.precise != 0, a);
        if (a.density > 1e-6f) {
          const float sa = density_alpha(ph.dx, len3(pos - prev), a.density);
          light = 1.f;
          if (R.shadows) light *= light_march(G, R, (prev + pos) * .5f, sun, suninv);
          light = R.ambient + light * ambInv;
          mix(smoke * light, sa, color, alpha);
        }
      }
    }
  }
  F3 pos = origin + dir * dSolid;
  const float bgAlpha = density_alpha(ph.dx, dSolid, 1e-6f);
  if (what == 1) {
    light = fmaxf(0.f, dot3(sdf_normal(g, ph, pos), sun));
    if (R.shadows) light *= light_march(G, R, pos, sun, suninv);
    light = R.ambient + light * ambInv;
    mix(f3(R.scene[0], R.scene[1], R.scene[2]) * light, 1.f - bgAlpha, color, alpha);
  }
  if (what == 2) {
    pos.y = 0.f;
    light = floorLight;
    if (R.shadows) light *= light_march(G, R, pos, sun, suninv);
    light = R.ambient + light * ambInv;
    light *= 1.f + .1f * fmodf(fabsf(floorf(pos.x / g.gx) + floorf(pos.z / g.gx)), 2.f);
    mix(f3(R.floor_[0], R.floor_[1], R.floor_[2]) * light, 1.f - bgAlpha, color, alpha);
  }
  if (what == 3) {
    pos.z = sliceZ;
    G.sample(pos, R.precise != 0, a);
    if (R.channel == CH_DENSITY) mix(f3(a.density * 1e2f, 0.f, 0.f), 1.f, color, alpha);
    if (R.channel == CH_VELOCITY) {
      const float v = G.vel_len(a) * 1e-1f;
      mix(f3(v - 2.f, v - 1.f, v), 1.f, color, alpha);
    }
    if (R.channel == CH_RESOLUTION) {
      const float c = (float)((a.ix / 4 + a.iy / 4) % 2);
      mix(f3(c, c, c), 1.f, color, alpha);
    }
    if (R.channel == CH_FLUIDITY) {
      const float f = G.fluid(a);
      mix(f3(f, f, f), 1.f, color, alpha);
    }
  }
  return make_float4(color.x, color.y, color.z, alpha);
}

// k_dcgrid_render camera (dcgrid_rendering.cu:58-92)
template <class Grid> __device__ float4 render_pixel(const Grid &G, const RenderP &R, int x, int y) {
  const float cx = .5f * R.width, cy = .5f * R.height;
  const float s = R.fov / fmaxf(cx, cy);
  const float step = 1.f / (float)R.aa;
  const F3 origin = f3(R.eye[0], R.eye[1], R.eye[2]) * G.ph().rdx;
  const F3 sun = f3(R.sun[0], R.sun[1], R.sun[2]);
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  for (float dx = 0; dx < 1.f; dx += step)
    for (float dy = 0; dy < 1.f; dy += step) {
      const F3 v = normalize3(f3((x + dx - cx) * s, (y + dy - cy) * s, 1.f));
      const F3 dir = f3(v.x, v.z * R.eye_dir[1] - v.y * R.eye_dir[2], v.y * R.eye_dir[1] + v.z * R.eye_dir[2]);
      const float4 c = ray_march(G, R, origin, dir, sun);
      acc.x += c.x; acc.y += c.y; acc.z += c.z; acc.w += c.w;
    }
  const float n = step * step;
  return make_float4(acc.x * n, acc.y * n, acc.z * n, acc.w * n);
}

__global__ void __launch_bounds__(256) k_render_adaptive(const __grid_constant__ Dev D, const __grid_constant__ RenderP R,
                                                         float4 *out) {
  const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
  if (x >= R.width || y >= R.height) return;
  out[(size_t)y * R.width + x] = render_pixel(AdaptiveGrid{D}, R, x, y);
}
__global__ void __launch_bounds__(256) k_render_uniform(const __grid_constant__ UDev U, const __grid_constant__ RenderP R,
                                                        float4 *out) {
  const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
  if (x >= R.width || y >= R.height) return;
  out[(size_t)y * R.width + x] = render_pixel(UniformGridR{U}, R, x, y);
}

}  // namespace

void launch_render_adaptive(const Dev &D, const RenderP &R, float4 *out, cudaStream_t st) {
  const dim3 grid((unsigned)((R.width + 15) / 16), (unsigned)((R.height + 15) / 16));
  k_render_adaptive<<<grid, 256, 0, st>>>(D, R, out);
}
void launch_render_uniform(const UDev &U, const RenderP &R, float4 *out, cudaStream_t st) {
  const dim3 grid((unsigned)((R.width + 15) / 16), (unsigned)((R.height + 15) / 16));
  k_render_uniform<<<grid, 256, 0, st>>>(U, R, out);
}

}  // namespace dcg
